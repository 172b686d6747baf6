"""X-ray tube excitation spectra (host pre-step).

``ebel`` wraps ``xmi_tube_ebel`` (the library's restatement of
src/xmi_ebel.F90:115-521: Ebel's model of a tube's continuum and K/L lines,
window and filter attenuation, optional transmission-efficiency profile) and
returns the spectrum as the input's continuous points and discrete lines.

``rh_tube_40kv`` builds the excitation of the production workload with it: a
rhodium anode at 40 kV behind a 125 um Be window, electrons at 60 degrees,
take-off at 20 degrees, continuum in ``n_intervals`` intervals over 1-40 keV,
plus the Rh K and L lines.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .simulation import ContinuousPoint, DiscreteLine, XmiError


def _xrl():
    """The library with the prototypes of its atomic data functions."""
    lib = abi.load()
    for name in ("xrl_CS_Total_Kissel", "xrl_LineEnergy", "xrl_RadRate", "xrl_FluorYield", "xrl_EdgeEnergy"):
        getattr(lib, name).restype = C.c_double
    lib.xrl_CS_Total_Kissel.argtypes = [C.c_int, C.c_double]
    lib.xrl_LineEnergy.argtypes = [C.c_int, C.c_int]
    lib.xrl_RadRate.argtypes = [C.c_int, C.c_int]
    lib.xrl_FluorYield.argtypes = [C.c_int, C.c_int]
    lib.xrl_EdgeEnergy.argtypes = [C.c_int, C.c_int]
    lib.xrl_prepare.argtypes = [C.c_int]
    return lib


def _layer(Z: int, density: float, thickness: float):
    z = (C.c_int * 1)(Z)
    w = (C.c_double * 1)(1.0)
    lay = abi.XmiLayer(1, C.cast(z, abi.c_int_p), C.cast(w, abi.c_double_p), density, thickness)
    return lay, (z, w)


def ebel(anode: tuple, voltage: float, current: float = 1.0, angle_electron: float = 60.0,
         angle_xray: float = 20.0, delta_energy: float = 0.1, solid_angle: float = 1e-4,
         window: tuple | None = None, filter: tuple | None = None, transmission: bool = False,
         efficiencies: tuple | None = None):
    """anode/window/filter: (Z, density g/cm3, thickness cm); efficiencies:
    (energies, values).  Returns (continuous points, discrete lines)."""
    lib = abi.load()
    keep = []
    layers = []
    for spec in (anode, window, filter):
        if spec is None:
            layers.append(None)
        else:
            lay, k = _layer(*spec)
            keep.append((lay, k))
            layers.append(C.pointer(lay))
    ne = 0
    ep = vp = None
    if efficiencies is not None:
        e = np.ascontiguousarray(efficiencies[0], dtype=np.float64)
        v = np.ascontiguousarray(efficiencies[1], dtype=np.float64)
        keep.append((e, v))
        ne, ep, vp = len(e), e.ctypes.data_as(abi.c_double_p), v.ctypes.data_as(abi.c_double_p)
    out = C.POINTER(abi.XmiExcitation)()
    if lib.xmi_tube_ebel(layers[0], layers[1], layers[2], voltage, current, angle_electron, angle_xray,
                         delta_energy, solid_angle, 1 if transmission else 0, ne, ep, vp, C.byref(out)) != 1:
        raise XmiError("xmi_tube_ebel failed: " + abi.last_error())
    exc = out.contents
    cont = [ContinuousPoint(exc.continuous[i].energy, exc.continuous[i].horizontal_intensity,
                            exc.continuous[i].vertical_intensity) for i in range(exc.n_continuous)]
    lines = [DiscreteLine(exc.discrete[i].energy, exc.discrete[i].horizontal_intensity,
                          exc.discrete[i].vertical_intensity) for i in range(exc.n_discrete)]
    for p in (exc.continuous, exc.discrete):
        if p:
            lib.xmi_free(C.cast(p, C.c_void_p))
    lib.xmi_free(C.cast(out, C.c_void_p))
    return cont, lines


def read_transmission_efficiency(path: str):
    """xmi_transmission_efficiency_read: (energies, efficiencies)."""
    lib = abi.load()
    n = C.c_size_t(0)
    e, v = abi.c_double_p(), abi.c_double_p()
    if lib.xmi_transmission_efficiency_read(path.encode(), C.byref(n), C.byref(e), C.byref(v)) != 1:
        raise XmiError(abi.last_error())
    out = (np.ctypeslib.as_array(e, (n.value,)).copy(), np.ctypeslib.as_array(v, (n.value,)).copy())
    lib.xmi_free(C.cast(e, C.c_void_p))
    lib.xmi_free(C.cast(v, C.c_void_p))
    return out


def rh_tube_40kv(n_intervals: int = 400, kv: float = 40.0, window_um: float = 125.0, current_ma: float = 1.0):
    """Rh anode (12.41 g/cm3, 1 cm) at kv behind window_um of Be (1.848
    g/cm3): n_intervals continuum intervals from 1 keV to kv (the step is
    chosen so that Ebel's grid, which ends on the tube voltage, has exactly
    n_intervals + 1 points) and the Rh K/L lines."""
    delta = (kv - 1.0) / (n_intervals - 0.5)
    return ebel((45, 12.41, 1.0), kv, current=current_ma, delta_energy=delta,
                window=(4, 1.848, window_um * 1e-4))
