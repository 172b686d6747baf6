"""X-ray tube spectra (xmi_tube_ebel, src/xmi_ebel.F90:115-521) and the
transmission-efficiency reader: the setups of the reference's
tests/test-ebel.c, the grid and line-selection rules of the model, the
window/filter attenuation and the natural cubic spline.  Host code only."""
import math
from pathlib import Path

import numpy as np
import pytest

from xmimsim_gb300 import tube
from xmimsim_gb300.simulation import XmiError

GOLDEN = Path(__file__).resolve().parent / "golden"
AG = (47, 10.5, 1.0)          # anode of tests/test-ebel.c: Ag, 1 cm
BE = (4, 1.848, 1e-4)         # 1 um Be window
C_FILTER = (6, 2.26, 1e-3)    # 10 um carbon filter


def run(**kw):
    args = dict(anode=AG, voltage=9.0, current=1.0, angle_electron=45.0, angle_xray=45.0, delta_energy=0.1,
                solid_angle=0.1)
    args.update(kw)
    return tube.ebel(**args)


@pytest.mark.parametrize("window,filt,eff", [(None, None, False), (BE, None, False), (BE, C_FILTER, False),
                                             (BE, C_FILTER, True)])
def test_reference_setups_succeed(window, filt, eff):
    """/ebel/good-* of tests/test-ebel.c: every setup returns a spectrum."""
    efficiencies = tube.read_transmission_efficiency(str(GOLDEN / "transmission_efficiency.txt")) if eff else None
    cont, lines = run(window=window, filter=filt, efficiencies=efficiencies)
    I = np.array([c.horizontal_intensity for c in cont])
    assert np.isfinite(I).all() and (I >= 0).all() and I.max() > 0
    assert all(l.horizontal_intensity > 0 and l.horizontal_intensity == l.vertical_intensity for l in lines)


def test_missing_transmission_file_is_an_error():
    """/ebel/bad-with-window-with-filter-with-efficiency."""
    with pytest.raises(XmiError):
        tube.read_transmission_efficiency("non-existent-file.txt")


def test_energy_grid_and_line_selection():
    """Intervals from 1 keV in steps of delta, the last point on the tube
    voltage (one extra point when the voltage is not a multiple of delta);
    at 9 kV the Ag K shell (25.5 keV) is not ionised: only L lines, all
    above 1 keV and below the voltage."""
    cont, lines = run()
    E = np.array([c.energy for c in cont])
    assert len(E) == math.floor((9.0 - 1.0) / 0.1) + 1
    assert E[0] == 1.0 and E[-1] == 9.0 and np.allclose(np.diff(E[:-1]), 0.1)
    cont2, _ = run(delta_energy=0.35)  # 9 / 0.35 is not an integer
    assert len(cont2) == math.floor((9.0 - 1.0) / 0.35) + 2 and cont2[-1].energy == 9.0
    assert lines and all(1.0 < l.energy < 9.0 for l in lines)
    assert all(l.energy < 4.0 for l in lines)  # Ag L lines only
    _, lines_k = run(voltage=40.0)
    assert any(l.energy > 20.0 for l in lines_k)  # Ag K lines once the K edge is exceeded


def test_window_and_filter_attenuate_as_the_model():
    """A window multiplies each interval by exp(-rho t mu) at the interval's
    middle, a filter at its start; lines at their energy -- ratios of two
    runs are those transmissions, so they are below 1, increase with energy
    above 1 keV, and the filter's ratio is the window-only run's times a
    second transmission."""
    c0, l0 = run()
    c1, l1 = run(window=BE)
    c2, l2 = run(window=BE, filter=C_FILTER)
    I0, I1, I2 = (np.array([c.horizontal_intensity for c in cc]) for cc in (c0, c1, c2))
    m = I0 > 0
    t1, t2 = I1[m] / I0[m], I2[m] / I1[m]
    assert (t1 < 1).all() and (t2 < 1).all()
    assert (np.diff(t1) > -1e-12).all() and (np.diff(t2) > -1e-12).all()
    for a, b in zip(l0, l1):
        assert a.energy == b.energy and b.horizontal_intensity < a.horizontal_intensity


def test_transmission_efficiency_spline():
    """The efficiency profile scales the spectrum by a natural cubic spline
    through the file's points: at a knot energy the factor is the knot's
    value."""
    e, v = tube.read_transmission_efficiency(str(GOLDEN / "transmission_efficiency.txt"))
    assert len(e) == 10 and e[0] == 0.5 and v[-1] == 0.93
    c0, _ = run(voltage=9.0, delta_energy=1.0)
    c1, _ = run(voltage=9.0, delta_energy=1.0, efficiencies=(e, v))
    for a, b in zip(c0, c1):
        if a.energy in (1.0, 2.0, 3.0, 5.0, 8.0) and a.horizontal_intensity > 0:
            k = list(e).index(a.energy)
            assert b.horizontal_intensity == pytest.approx(a.horizontal_intensity * v[k], rel=1e-12)
