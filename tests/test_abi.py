"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: these run without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(xmi_\w+)\s*\(", text, flags=re.M):
            if m.group(0).startswith("static"):
                continue  # inline helpers of the data-format header, not exports
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("xmi_main_msim", "xmi_solid_angle_calculation", "xmi_detector_convolute_all",
                "xmi_detector_convolute_spectrum", "xmi_detector_convolute_history", "xmi_escape_ratios_calculation",
                "xmi_input_C2F", "xmi_init_input", "xmi_init_from_hdf5", "xmi_solid_angle_calculation_cuda",
                "xmi_detector_convolute_all_custom"):
        assert ref in names


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(name):
    from xmimsim_gb300 import abi
    lib = abi.load()
    assert hasattr(lib, name), name


def test_hits_per_single_variable_exported():
    from xmimsim_gb300 import abi
    v = C.c_long.in_dll(abi.load(), "hits_per_single")
    assert v.value == 5000


def test_no_gpu_fails_loudly_without_device():
    """Without a CUDA device every compute entry point returns an error
    (no CPU fallback)."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from xmimsim_gb300 import Simulation, XmiError, configs
    sim = Simulation(configs.config1(n_photons_line=10), options=configs.C1_OPTIONS)
    with pytest.raises(XmiError):
        sim.solid_angle()
    sim.close()
