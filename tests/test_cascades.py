"""Analog cascades (variance reduction off) on the CPU: the Auger and
radiative cascades of src/xmi_main.F90:2413-4783 in the oracle.  The
reference holds no vectors for them, so these are property checks on the
oracle that the GPU parity tests then compare against:
- a radiative cascade leaves its parent's trajectory untouched (the
  offspring draws from its own streams), so histories of lines that no
  cascade feeds are identical with and without it, while the lines of the
  shells the vacancies move to gain;
- an Auger cascade turns photons that would be absorbed into fluorescence
  photons of the new vacancies, so L lines gain;
- the stand-in Auger transition probabilities of each K/L vacancy sum to 1
  where the shells exist, in xraylib's transition order."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))

from oracle import oracle_api as O  # noqa: E402
from xmimsim_gb300 import Layer, Simulation, abi, configs  # noqa: E402


def _spec(n=60000):
    spec = configs.config1(n_photons_line=n)
    spec.layers = [Layer([82, 26, 8], [0.3, 0.4, 0.3], 6.0, 0.02)]
    spec.reference_layer = 1
    spec.n_interactions_trajectory = 3
    spec.p_detector_window = (0.0, 1.0, 100.0)
    spec.discrete[0].energy = 90.0  # above the Pb K edge
    return spec


def _run(auger, radiative, n=60000):
    spec = _spec(n)
    sim = Simulation(spec, options=dict(configs.C1_OPTIONS, use_variance_reduction=0, use_cascade_auger=auger,
                                        use_cascade_radiative=radiative))
    sim.prepare()
    out = O.msim(sim.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels)
    sim.close()
    return out


def test_auger_rates_sum_to_one():
    import ctypes as C
    lib = abi.load()
    lib.xrl_AugerRate.restype = C.c_double
    lib.xrl_AugerRate.argtypes = [C.c_int, C.c_int]
    for Z in (26, 47, 82):
        k = sum(lib.xrl_AugerRate(Z, t) for t in range(240))
        assert k == pytest.approx(1.0, rel=1e-12)
        for s in range(3):
            v = sum(lib.xrl_AugerRate(Z, 240 + 135 * s + t) for t in range(135))
            assert v == pytest.approx(1.0, rel=1e-12)
    # a K vacancy of oxygen: L transitions only, still a distribution
    assert sum(lib.xrl_AugerRate(8, t) for t in range(240)) == pytest.approx(1.0, rel=1e-12)
    assert all(lib.xrl_AugerRate(8, t) == 0.0 for t in range(30 * 3, 240))  # no M vacancies in O


def test_radiative_cascade_only_adds_offspring():
    base, rad = _run(0, 0), _run(0, 1)
    b, r = base["brute"], rad["brute"]
    pb = 82 - 1
    # Pb K lines of the first order come from parents alone, which the
    # offspring never perturb (equal up to the order of the additions)
    k_lines = slice(0, 29)
    np.testing.assert_allclose(r[pb, k_lines, 0], b[pb, k_lines, 0], rtol=1e-12)
    # Pb L lines gain from K vacancies moving to L (first order: offspring
    # tallied at the parent's interaction order)
    l_lines = slice(29, 113)
    assert r[pb, l_lines, 0].sum() > b[pb, l_lines, 0].sum() * 1.01
    assert r.sum() > b.sum()


def test_auger_cascade_adds_l_lines():
    base, aug = _run(0, 0), _run(1, 0)
    pb = 82 - 1
    l_lines = slice(29, 113)
    assert aug["brute"][pb, l_lines, 0].sum() > base["brute"][pb, l_lines, 0].sum() * 1.01
    # first-order K lines come from photons whose K vacancy fluoresced: untouched
    np.testing.assert_allclose(aug["brute"][pb, 0:29, 0], base["brute"][pb, 0:29, 0], rtol=1e-12)
