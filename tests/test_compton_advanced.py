"""Advanced Compton scattering (use_advanced_compton = 1) on the CPU: the
momentum kinematics (src/xmi_aux_f.F90:1951-2074), the per-shell Compton
profile tables (src/xmi_data_f.F90:1124-1230), and the oracle's transport
and estimator with them against the default Doppler path.  The reference's
own tests hold no vectors for this path, so these are property checks: Qimax
is the momentum at which the whole energy above the binding energy is
transferred, E(Q) inverts Q(E), the tables are monotone with the reference's
end values, and the shell mixture keeps the element's Compton weight."""
import math
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))

from oracle import oracle_api as O  # noqa: E402
from xmimsim_gb300 import Layer, Simulation, configs  # noqa: E402

MEC2 = 510.998928


def test_qimax_is_the_momentum_of_the_full_transfer():
    for E in (2.0, 8.04, 17.4, 59.3, 150.0):
        for Ii in (0.0, 0.01, 0.5, 1.5):
            for th in np.linspace(0.05, math.pi - 0.05, 13):
                q = O.compton_qimax(E, Ii, th)
                assert q == pytest.approx(O.compton_q_from_energy(E, E - Ii, th), rel=1e-12, abs=1e-12)
    assert O.compton_qimax(5.0, 7.1, 1.0) == 0.0  # binding energy above the photon energy


def test_energy_from_q_inverts_q_from_energy():
    worst = 0.0
    for E in (1.5, 5.0, 17.4, 60.0, 150.0):
        for th in np.linspace(0.1, math.pi - 0.01, 19):
            prev = 0.0
            for Q in np.linspace(-99.0, 99.0, 199):
                if abs(Q) < 0.01:
                    continue
                e2, err = O.compton_energy_from_q(E, Q, th)
                assert err == 0
                assert e2 > prev  # the scattered energy grows with Q
                prev = e2
                worst = max(worst, abs(O.compton_q_from_energy(E, e2, th) - Q) / abs(Q))
    assert worst < 1e-8


def test_energy_from_q_special_cases():
    E, th = 20.0, 1.2
    compton = E / (1.0 + E * (1.0 - math.cos(th)) / MEC2)
    assert O.compton_energy_from_q(E, 5e-5, th)[0] == pytest.approx(compton, rel=1e-15)
    assert O.compton_energy_from_q(E, 3.0, 1e-5) == (0.0, 0)  # theta ~ 0: no scattering
    # positive Q gives energies above the Compton line, negative below
    assert O.compton_energy_from_q(E, 2.0, th)[0] > compton > O.compton_energy_from_q(E, -2.0, th)[0]


def _grid(sim, n=48, hits=1500):
    from test_oracle import _oracle_grid
    _oracle_grid(sim, n, n, hits)


def _heavy_spec(n=3000):
    spec = configs.config1(n_photons_line=n)
    spec.layers = [Layer([82, 8, 26], [0.6, 0.3, 0.1], 5.0, 0.01)]
    spec.reference_layer = 1
    return spec


def test_profile_tables():
    spec = _heavy_spec()
    sim = Simulation(spec, options=dict(configs.C1_OPTIONS, use_advanced_compton=1, use_default_seeds=1))
    _grid(sim)
    sim.prepare()
    ptr = sim.bundle_ptr()
    Qs = 100.0 * np.arange(10001) / 10000.0
    cs = 0.5 * np.arange(10001) / 10000.0
    zs = []
    for e in range(3):
        shells, occ, edge = O.compton_shells(ptr, e)
        assert shells[0] == 0 and np.all(np.diff(shells) > 0)
        zs.append(occ.sum())
        assert edge[0] == edge.max() > 0  # K is the most bound shell
        for k in range(len(shells)):
            cdf, qinv = O.compton_rows(ptr, e, k)
            assert cdf[0] == 0.0 and cdf[-1] == 0.5 and np.all(np.diff(cdf) >= 0)
            assert qinv[0] == 0.0 and qinv[-1] == 100.0 and np.all(np.diff(qinv) >= 0)
            # the inverse table inverts the forward table (the trapezoid rule of
            # the forward table against the exact integral of the inverse)
            back = np.interp(qinv[1:-1], Qs, cdf)
            assert np.abs(back - cs[1:-1]).max() < 2e-4
    # the occupancies add up to Z; the stand-in configuration model keeps one
    # electron in every shell bound at that Z, a little above Z for heavy atoms
    for z, want in zip(sorted(zs), (8, 26, 82)):
        assert want <= z <= want + 2
    sim.close()


def test_transport_draw_follows_the_shell_mixture():
    """The transport's scattered energy: shells chosen by occupancy x cumulative
    profile, energies inside the kinematic range of the chosen shell."""
    spec = _heavy_spec()
    sim = Simulation(spec, options=dict(configs.C1_OPTIONS, use_advanced_compton=1, use_default_seeds=1))
    _grid(sim)
    sim.prepare()
    ptr = sim.bundle_ptr()
    pb = max(range(3), key=lambda e: O.compton_shells(ptr, e)[1].sum())  # lead
    E, th = 30.0, 1.7
    energies = []
    for pid in range(4000):
        e2, cdfs, err = O.compton_energy_advanced(ptr, pb, E, th, pid, 2)
        assert err == 0
        energies.append(e2)
    energies = np.array(energies)
    compton = E / (1.0 + E * (1.0 - math.cos(th)) / MEC2)
    assert np.all(energies > 0) and np.all(energies < E)
    # Doppler broadening around the Compton line: median near it, spread of a few percent
    assert np.median(energies) == pytest.approx(compton, rel=0.02)
    assert 0.002 < np.std(energies) / compton < 0.2
    sim.close()


def test_oracle_advanced_compton_keeps_the_compton_weight():
    """The per-shell estimator splits each element's Compton weight over its
    shells (shares summing to 1), so its Compton history differs from the
    default path's only through the escape probability at the shell energies;
    Rayleigh and fluorescence histories of the first order are unchanged."""
    spec = _heavy_spec(4000)
    out = []
    for adv in (0, 1):
        sim = Simulation(spec, options=dict(configs.C1_OPTIONS, use_advanced_compton=adv, use_default_seeds=1))
        _grid(sim)
        sim.prepare()
        out.append(O.msim(sim.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels))
        sim.close()
    d, a = out
    c_d, c_a = d["var_red"][:, 384, 0].sum(), a["var_red"][:, 384, 0].sum()
    assert c_a == pytest.approx(c_d, rel=5e-3)
    np.testing.assert_allclose(a["var_red"][:, :384, 0], d["var_red"][:, :384, 0], rtol=1e-12, atol=0)
    # the spectra differ in the shape of the Compton peak, not in its area
    assert not np.array_equal(a["channels"][1], d["channels"][1])
