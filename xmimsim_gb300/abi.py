"""ctypes mirror of the engine's C-ABI (include/xmimsim_gb300.h).

The structures reproduce the reference's C data model
(include/xmi_data_structs.h of XMI-MSIM) field for field; the functions are
the library's exported entry points.  Loading fails loudly when the shared
library has not been built -- there is no Python fallback for any compute.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libxmimsim_gb300.so"

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)


class XmiGeneral(C.Structure):
    _fields_ = [("version", C.c_float), ("outputfile", C.c_char_p), ("n_photons_interval", C.c_long),
                ("n_photons_line", C.c_long), ("n_interactions_trajectory", C.c_int), ("comments", C.c_char_p)]


class XmiLayer(C.Structure):
    _fields_ = [("n_elements", C.c_int), ("Z", c_int_p), ("weight", c_double_p), ("density", C.c_double),
                ("thickness", C.c_double)]


class XmiComposition(C.Structure):
    _fields_ = [("n_layers", C.c_int), ("layers", C.POINTER(XmiLayer)), ("reference_layer", C.c_int)]


class XmiGeometry(C.Structure):
    _fields_ = [("d_sample_source", C.c_double), ("n_sample_orientation", C.c_double * 3),
                ("p_detector_window", C.c_double * 3), ("n_detector_orientation", C.c_double * 3),
                ("area_detector", C.c_double), ("collimator_height", C.c_double),
                ("collimator_diameter", C.c_double), ("d_source_slit", C.c_double), ("slit_size_x", C.c_double),
                ("slit_size_y", C.c_double)]


class XmiEnergyDiscrete(C.Structure):
    _fields_ = [("energy", C.c_double), ("horizontal_intensity", C.c_double), ("vertical_intensity", C.c_double),
                ("sigma_x", C.c_double), ("sigma_xp", C.c_double), ("sigma_y", C.c_double),
                ("sigma_yp", C.c_double), ("distribution_type", C.c_int), ("scale_parameter", C.c_double)]


class XmiEnergyContinuous(C.Structure):
    _fields_ = [("energy", C.c_double), ("horizontal_intensity", C.c_double), ("vertical_intensity", C.c_double),
                ("sigma_x", C.c_double), ("sigma_xp", C.c_double), ("sigma_y", C.c_double),
                ("sigma_yp", C.c_double)]


class XmiExcitation(C.Structure):
    _fields_ = [("n_discrete", C.c_int), ("discrete", C.POINTER(XmiEnergyDiscrete)), ("n_continuous", C.c_int),
                ("continuous", C.POINTER(XmiEnergyContinuous))]


class XmiAbsorbers(C.Structure):
    _fields_ = [("n_exc_layers", C.c_int), ("exc_layers", C.POINTER(XmiLayer)), ("n_det_layers", C.c_int),
                ("det_layers", C.POINTER(XmiLayer))]


class XmiDetector(C.Structure):
    _fields_ = [("detector_type", C.c_int), ("live_time", C.c_double), ("pulse_width", C.c_double),
                ("gain", C.c_double), ("zero", C.c_double), ("fano", C.c_double), ("noise", C.c_double),
                ("nchannels", C.c_int), ("n_crystal_layers", C.c_int), ("crystal_layers", C.POINTER(XmiLayer))]


class XmiInput(C.Structure):
    _fields_ = [("general", C.POINTER(XmiGeneral)), ("composition", C.POINTER(XmiComposition)),
                ("geometry", C.POINTER(XmiGeometry)), ("excitation", C.POINTER(XmiExcitation)),
                ("absorbers", C.POINTER(XmiAbsorbers)), ("detector", C.POINTER(XmiDetector))]


class XmiCounts(C.Structure):
    _fields_ = [("counts", C.c_double), ("interaction_number", C.c_int)]


class XmiFluorescenceLine(C.Structure):
    _fields_ = [("line_type", C.c_char_p), ("energy", C.c_double), ("total_counts", C.c_double),
                ("n_interactions", C.c_int), ("interactions", C.POINTER(XmiCounts))]


class XmiFluorescenceLineCounts(C.Structure):
    _fields_ = [("atomic_number", C.c_int), ("total_counts", C.c_double), ("n_lines", C.c_int),
                ("lines", C.POINTER(XmiFluorescenceLine))]


class XmiOutput(C.Structure):
    _fields_ = [("version", C.c_float), ("inputfile", C.c_char_p), ("outputfile", C.c_char_p),
                ("input", C.POINTER(XmiInput)), ("brute_force_history", C.POINTER(XmiFluorescenceLineCounts)),
                ("var_red_history", C.POINTER(XmiFluorescenceLineCounts)), ("nbrute_force_history", C.c_int),
                ("nvar_red_history", C.c_int), ("channels_conv", C.POINTER(C.POINTER(C.c_double))),
                ("channels_unconv", C.POINTER(C.POINTER(C.c_double))), ("ninteractions", C.c_int),
                ("use_zero_interactions", C.c_int)]


class XmiMainOptions(C.Structure):
    _fields_ = [("use_M_lines", C.c_int), ("use_cascade_auger", C.c_int), ("use_cascade_radiative", C.c_int),
                ("use_variance_reduction", C.c_int), ("use_sum_peaks", C.c_int), ("use_escape_peaks", C.c_int),
                ("escape_ratios_mode", C.c_int), ("verbose", C.c_int), ("use_poisson", C.c_int),
                ("use_gpu", C.c_int), ("omp_num_threads", C.c_int), ("extra_verbose", C.c_int),
                ("custom_detector_response", C.c_char_p), ("use_advanced_compton", C.c_int),
                ("use_default_seeds", C.c_int)]


class XmiSolidAngle(C.Structure):
    _fields_ = [("solid_angles", c_double_p), ("grid_dims_r_n", C.c_long), ("grid_dims_theta_n", C.c_long),
                ("grid_dims_r_vals", c_double_p), ("grid_dims_theta_vals", c_double_p),
                ("xmi_input_string", C.c_char_p)]


class XmiEscapeRatios(C.Structure):
    _fields_ = [("n_elements", C.c_int), ("n_fluo_input_energies", C.c_int),
                ("n_compton_input_energies", C.c_int), ("n_compton_output_energies", C.c_int), ("Z", c_int_p),
                ("fluo_escape_ratios", c_double_p), ("fluo_escape_input_energies", c_double_p),
                ("compton_escape_ratios", c_double_p), ("compton_escape_input_energies", c_double_p),
                ("compton_escape_output_energies", c_double_p), ("xmi_input_string", C.c_char_p)]


class XmiEscapeRatiosOptions(C.Structure):
    _fields_ = [("n_input_energies", C.c_long), ("n_compton_output_energies", C.c_long),
                ("n_photons", C.c_long), ("input_energy_min", C.c_double), ("input_energy_delta", C.c_double),
                ("compton_output_energy_min", C.c_double), ("compton_output_energy_delta", C.c_double)]


class XmiGpuOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("use_surrogate", C.c_int), ("surrogate_tolerance", C.c_double),
                ("threads_per_block", C.c_int), ("blocks_per_sm", C.c_int), ("seed", C.c_ulonglong),
                ("solid_angle_stream", C.c_int), ("queue_events", C.c_longlong),
                ("grid_nr", C.c_int), ("grid_nt", C.c_int), ("overlap_chunks", C.c_int),
                ("estimator_blocks_per_sm", C.c_int)]


# the atomic data source table (xmi_atomic_data): entry name -> argument types
ATOMIC_DATA_ENTRIES = [
    ("AtomicWeight", [C.c_int]), ("EdgeEnergy", [C.c_int, C.c_int]), ("ElectronConfig", [C.c_int, C.c_int]),
    ("LineEnergy", [C.c_int, C.c_int]), ("RadRate", [C.c_int, C.c_int]), ("FluorYield", [C.c_int, C.c_int]),
    ("AugerYield", [C.c_int, C.c_int]), ("CosKronTransProb", [C.c_int, C.c_int]), ("AugerRate", [C.c_int, C.c_int]),
    ("AugerVacancies", [C.c_int, C.c_int, C.c_int]), ("CS_Total_Kissel", [C.c_int, C.c_double]),
    ("CS_Photo_Total", [C.c_int, C.c_double]), ("CS_Photo_Partial", [C.c_int, C.c_int, C.c_double]),
    ("CS_Rayl", [C.c_int, C.c_double]), ("CS_Compt", [C.c_int, C.c_double]), ("FF_Rayl", [C.c_int, C.c_double]),
    ("SF_Compt", [C.c_int, C.c_double]), ("DCS_Rayl", [C.c_int, C.c_double, C.c_double]),
    ("DCS_Compt", [C.c_int, C.c_double, C.c_double]), ("ComptonProfile", [C.c_int, C.c_double]),
]
ATOMIC_DATA_FUNC = {name: C.CFUNCTYPE(C.c_double, *args) for name, args in ATOMIC_DATA_ENTRIES}
PREPARE_FUNC = C.CFUNCTYPE(None, C.c_int)


class XmiAtomicData(C.Structure):
    _fields_ = [("name", C.c_char_p)] + [(name, ATOMIC_DATA_FUNC[name]) for name, _ in ATOMIC_DATA_ENTRIES] + \
        [("prepare", PREPARE_FUNC)]


# exported symbols and their prototypes (name -> (restype, argtypes))
PROTOTYPES = {
    "xmi_input_init_empty": (C.POINTER(XmiInput), []),
    "xmi_input_free": (None, [C.POINTER(XmiInput)]),
    "xmi_input_copy": (None, [C.POINTER(XmiInput), C.POINTER(C.POINTER(XmiInput))]),
    "xmi_main_options_new": (C.POINTER(XmiMainOptions), []),
    "xmi_main_options_free": (None, [C.POINTER(XmiMainOptions)]),
    "xmi_free": (None, [C.c_void_p]),
    "xmi_gpu_last_error": (C.c_char_p, []),
    "xmi_gpu_default_options": (None, [C.POINTER(XmiGpuOptions)]),
    "xmi_input_C2F": (C.c_int, [C.POINTER(XmiInput), C.POINTER(C.c_void_p)]),
    "xmi_free_input_F": (None, [C.POINTER(C.c_void_p)]),
    "xmi_init_input": (C.c_int, [C.POINTER(C.c_void_p)]),
    "xmi_init_input_escape_ratios": (C.c_int, [C.POINTER(C.c_void_p)]),
    "xmi_init_from_hdf5": (C.c_int, [C.c_char_p, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(XmiMainOptions)]),
    "xmi_update_input_from_hdf5": (C.c_int, [C.c_void_p, C.c_void_p]),
    "xmi_free_hdf5_F": (None, [C.POINTER(C.c_void_p)]),
    "xmi_gpu_set_options": (C.c_int, [C.c_void_p, C.POINTER(XmiGpuOptions)]),
    "xmi_solid_angle_calculation": (None, [C.c_void_p, C.POINTER(C.POINTER(XmiSolidAngle)), C.c_char_p,
                                           C.POINTER(XmiMainOptions)]),
    "xmi_solid_angle_calculation_cuda": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(XmiSolidAngle)), C.c_char_p,
                                                   C.POINTER(XmiMainOptions)]),
    "xmi_free_solid_angle": (None, [C.POINTER(XmiSolidAngle)]),
    "xmi_main_msim": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(c_double_p), C.POINTER(XmiMainOptions),
                                C.POINTER(c_double_p), C.POINTER(c_double_p), C.POINTER(XmiSolidAngle)]),
    "xmi_detector_convolute_spectrum": (None, [C.c_void_p, c_double_p, C.POINTER(c_double_p),
                                               C.POINTER(XmiMainOptions), C.POINTER(XmiEscapeRatios), C.c_int]),
    "xmi_detector_convolute_all": (None, [C.c_void_p, C.POINTER(c_double_p), C.POINTER(c_double_p), c_double_p,
                                          c_double_p, C.POINTER(XmiMainOptions), C.POINTER(XmiEscapeRatios), C.c_int,
                                          C.c_int]),
    "xmi_detector_convolute_all_custom": (None, [C.c_void_p, C.POINTER(c_double_p), C.POINTER(c_double_p),
                                                 c_double_p, c_double_p, C.POINTER(XmiMainOptions),
                                                 C.POINTER(XmiEscapeRatios), C.c_int, C.c_int]),
    "xmi_detector_convolute_history": (None, [C.c_void_p, c_double_p, C.POINTER(XmiMainOptions)]),
    "xmi_detector_convolute_spectrum_noalloc": (C.c_int, [C.c_void_p, c_double_p, c_double_p,
                                                          C.POINTER(XmiMainOptions)]),
    "xmi_get_default_escape_ratios_options": (XmiEscapeRatiosOptions, []),
    "xmi_escape_ratios_calculation": (None, [C.POINTER(XmiInput), C.POINTER(C.POINTER(XmiEscapeRatios)), C.c_char_p,
                                             C.c_char_p, C.POINTER(XmiMainOptions), XmiEscapeRatiosOptions]),
    "xmi_free_escape_ratios": (None, [C.POINTER(XmiEscapeRatios)]),
    "xmi_gpu_bundle": (C.c_void_p, [C.c_void_p]),
    "xmi_gpu_prepare_run": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(XmiMainOptions), C.c_int,
                                      C.POINTER(XmiSolidAngle)]),
    "xmi_gpu_last_timing": (C.c_int, [c_double_p, c_double_p, c_int_p]),
    "xmi_gpu_last_phases": (C.c_int, [c_double_p, c_double_p, c_double_p, C.POINTER(C.c_longlong)]),
    "xmi_gpu_set_replica": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "xmi_gpu_build_surrogate": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, c_double_p]),
    "xmi_gpu_surrogate_report": (C.c_int, [C.c_void_p, c_double_p]),
    "xmi_gpu_share_surrogate": (C.c_int, [C.c_void_p, C.c_void_p]),
    "xmi_gpu_surrogate_eval": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p, c_double_p,
                                         C.POINTER(C.c_int)]),
    "xmi_gpu_solid_angle_points": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p, C.c_int, C.c_int,
                                             C.c_ulonglong, c_double_p]),
    "xmi_gpu_last_graph": (C.c_int, [C.POINTER(C.c_int)]),
    "xmi_set_atomic_data": (C.c_int, [C.POINTER(XmiAtomicData)]),
    "xmi_output_raw2struct": (C.POINTER(XmiOutput), [C.POINTER(XmiInput), c_double_p, c_double_p,
                                                     C.POINTER(c_double_p), c_double_p, C.c_char_p, C.c_int]),
    "xmi_output_free": (None, [C.POINTER(XmiOutput)]),
    "xmi_output_write_to_xml_file": (C.c_int, [C.POINTER(XmiOutput), C.c_char_p, C.c_void_p]),
    "xmi_get_atomic_data": (C.POINTER(XmiAtomicData), []),
    "xmi_gpu_compton_kinematics": (C.c_int, [C.c_int, c_double_p, c_double_p, c_double_p, c_double_p,
                                             c_double_p]),
    "xmi_tube_ebel": (C.c_int, [C.POINTER(XmiLayer), C.POINTER(XmiLayer), C.POINTER(XmiLayer), C.c_double,
                                C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_size_t,
                                c_double_p, c_double_p, C.POINTER(C.POINTER(XmiExcitation))]),
    "xmi_transmission_efficiency_read": (C.c_int, [C.c_char_p, C.POINTER(C.c_size_t), C.POINTER(c_double_p),
                                                   C.POINTER(c_double_p)]),
    "xmi_gpu_escape_tables": (C.c_int, [C.POINTER(XmiInput), C.POINTER(XmiMainOptions), C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_void_p)]),
    "xmi_gpu_build_surrogate_points": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p, C.c_int, C.c_int,
                                                 C.c_int, c_double_p]),
    "xmi_gpu_sample_event_points": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(XmiMainOptions), C.c_double,
                                              C.c_int, c_double_p, c_double_p, C.POINTER(C.c_int)]),
    "xmi_gpu_autotune_batch": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                         C.POINTER(C.POINTER(XmiMainOptions)), C.POINTER(C.POINTER(XmiSolidAngle)),
                                         C.c_double, c_double_p]),
    "xmi_gpu_last_transfers": (C.c_int, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "xmi_gpu_last_surrogate": (C.c_int, [c_double_p, C.POINTER(C.c_longlong)]),
    "xmi_mlp_nparam": (C.c_int, []),
    "xmi_gpu_mlp_forward": (C.c_int, [C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "xmi_gpu_mlp_grad": (C.c_int, [C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float), c_double_p]),
    "xmi_gpu_mlp_train": (C.c_int, [C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.c_int, C.c_float, c_double_p]),
    "xmi_main_msim_batch": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                      C.POINTER(C.POINTER(XmiMainOptions)), C.POINTER(C.POINTER(XmiSolidAngle)),
                                      C.POINTER(c_double_p), C.POINTER(c_double_p), C.POINTER(c_double_p)]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libxmimsim_gb300.so (building it is ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else Path(os.environ.get("XMIMSIM_GB300_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build the CUDA engine first (python -c 'import __graft_entry__ as g; "
                           "g.build()'); there is no CPU fallback")
    lib = C.CDLL(str(p), mode=C.RTLD_GLOBAL)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    msg = load().xmi_gpu_last_error()
    return msg.decode() if msg else ""
