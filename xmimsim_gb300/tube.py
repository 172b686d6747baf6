"""X-ray tube excitation spectra (host pre-step).

``rh_tube_40kv`` builds the excitation of the production workload: a
rhodium-anode tube at 40 kV behind a 125 um Be window, discretised into
400 intervals over 1-40 keV, plus the Rh K and L lines.  The continuum
follows Kramers' law with the anode self-absorption factor of Ebel's model
(Ebel 1999, X-Ray Spectrom. 28, 255; the reference implements it in
src/xmi_ebel.F90:115-521) in simplified form; the characteristic lines carry
their intensity relative to the continuum at the line energy.  Attenuation
coefficients come from the engine library's atomic data model.
"""
from __future__ import annotations

import ctypes as C
import math

from . import abi
from .simulation import ContinuousPoint, DiscreteLine


def _xrl():
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


def rh_tube_40kv(n_intervals: int = 400, kv: float = 40.0, e_min: float = 1.0, window_um: float = 125.0,
                 current_ma: float = 1.0, takeoff_deg: float = 20.0):
    lib = _xrl()
    Z_anode, Z_be = 45, 4
    lib.xrl_prepare(Z_anode)
    lib.xrl_prepare(Z_be)
    rho_be, t_be = 1.85, window_um * 1e-4
    e_max = kv
    sin_t = math.sin(math.radians(takeoff_deg))

    def continuum(E):
        if E >= e_max:
            return 0.0
        kramers = 1.35e9 * current_ma * Z_anode * (e_max / E - 1.0)
        mu = lib.xrl_CS_Total_Kissel(Z_anode, E)
        # absorption of the emerging radiation in the anode (depth ~ rho z ~ 1e-4 g/cm2 scale)
        chi = mu / sin_t * 2.0e-4 * (e_max ** 1.6 - E ** 1.6) ** 0.5 / 10.0
        f_abs = (1.0 - math.exp(-2.0 * chi)) / (2.0 * chi) if chi > 1e-12 else 1.0
        win = math.exp(-rho_be * t_be * lib.xrl_CS_Total_Kissel(Z_be, E))
        return kramers * f_abs * win

    cont = []
    for i in range(n_intervals + 1):
        E = e_min + (e_max - e_min) * i / n_intervals
        I = continuum(E)
        cont.append(ContinuousPoint(E, I / 2.0, I / 2.0))
    lines = []
    # Rh K lines (KL2, KL3, KM2, KM3) and L3/L2 main lines
    for shell, line_ids in ((0, (2, 3, 5, 6)), (3, (89, 90)), (2, (63,))):
        edge = lib.xrl_EdgeEnergy(Z_anode, shell)
        if edge <= 0.0 or edge >= e_max:
            continue
        u0 = e_max / edge
        strength = 6.0e8 * current_ma * (u0 * math.log(u0) - u0 + 1.0) * lib.xrl_FluorYield(Z_anode, shell)
        for l in line_ids:
            El = lib.xrl_LineEnergy(Z_anode, l)
            rr = lib.xrl_RadRate(Z_anode, l)
            if El <= e_min or rr <= 0.0:
                continue
            win = math.exp(-rho_be * t_be * lib.xrl_CS_Total_Kissel(Z_be, El))
            I = strength * rr * win
            lines.append(DiscreteLine(El, I / 2.0, I / 2.0))
    return cont, lines
