"""Quantification loop of xmimsim-pymca (bin/xmimsim-pymca.c:597-820,
src/xmi_pymca.c:1647-1830) on the batched engine: the host rules on the CPU,
and on the GPU a closed loop -- measured intensities simulated from known
compositions are quantified back, several samples in one batch per
iteration."""
import math

import numpy as np
import pytest

from xmimsim_gb300 import Layer, configs, gpu_options
from xmimsim_gb300 import quant


def test_max_scale_table():
    assert quant.max_scale(1e-5) == 100.0
    assert quant.max_scale(0.0001) == 100.0
    assert quant.max_scale(0.005) == 10.0
    assert quant.max_scale(0.05) == 2.5
    assert quant.max_scale(0.2) == 1.5
    assert quant.max_scale(0.3) == 1.2
    assert quant.max_scale(0.45) == 1.1
    assert quant.max_scale(0.55) == 1.05
    assert quant.max_scale(0.65) == 1.025
    assert quant.max_scale(0.9) == 1.01


def test_layer_composition_rules():
    matrix = Layer([14, 8], [2.0, 2.0], 2.5, 0.1)  # un-normalised matrix weights
    w = np.array([0.05, 0.02])
    lay = quant.layer_composition(matrix, [26, 29], w)
    assert lay.Z == [8, 14, 26, 29]  # sorted by Z
    assert sum(lay.weight) == pytest.approx(1.0)
    assert lay.weight[2] == 0.05 and lay.weight[3] == 0.02
    assert lay.weight[0] == pytest.approx(0.5 * 0.93)
    # reference element of the matrix kept at its weight
    lay = quant.layer_composition(Layer([14, 8], [0.5, 0.5], 2.5, 0.1), [26], np.array([0.1]), reference=8,
                                  usematrix=True)
    d = dict(zip(lay.Z, lay.weight))
    assert d[8] == pytest.approx(0.5) and d[26] == pytest.approx(0.1) and d[14] == pytest.approx(0.4)
    # quantified weights above 1: those up to the largest are scaled to fill 1, the matrix gets nothing
    w = np.array([0.7, 0.6])
    lay = quant.layer_composition(matrix, [26, 29], w, k_exp=[1.0, 2.0], l_exp=[0.0, 0.0])
    d = dict(zip(lay.Z, lay.weight))
    assert d[14] == pytest.approx(0.0, abs=1e-15) and d[8] == pytest.approx(0.0, abs=1e-15)
    assert sum(lay.weight) == pytest.approx(1.0)
    assert w[0] == pytest.approx(0.4)  # updated in place: 0.7 * (1 - 0.6) / 0.7


def test_detector_absorption_bounds():
    spec = configs.config1(n_photons_line=10)
    a_fe = quant.detector_absorption(spec, 26, "KL3")
    a_si = quant.detector_absorption(spec, 14, "KL3")
    assert 0.0 < a_si < a_fe <= 1.0  # the Be window absorbs soft Si-K more than Fe-K


def _sample_spec(weights, n=60000):
    spec = configs.config1(n_photons_line=n)
    matrix = Layer([8, 14], [0.5, 0.4], 2.5, 0.1)
    lay = quant.layer_composition(matrix, [26, 29, 30], np.array(weights, dtype=np.float64))
    spec.layers = [spec.layers[0], lay]
    return spec, matrix


@pytest.mark.gpu
def test_closed_loop_recovers_known_compositions():
    """Three samples with known Fe/Cu/Zn weights: their K-alpha intensities
    simulated at the known composition (each with its own solid-angle grid)
    are quantified back from the start concentration 1e-4, all three in one
    batch per iteration; the recovered weights match within 1% and the loop
    ends on the reference's convergence test."""
    from xmimsim_gb300 import Simulation
    truths = [[0.05, 0.03, 0.02], [0.01, 0.10, 0.004], [0.20, 0.002, 0.05]]
    opts = dict(configs.C1_OPTIONS, use_escape_peaks=0)
    gpu = gpu_options(precision=1, seed=0x5EED0001)
    samples = []
    for t in truths:
        spec, matrix = _sample_spec(t)
        sim = Simulation(spec, options=opts, gpu=gpu)
        sim.solid_angle()
        out = sim.msim()
        k = [quant._simulated_alpha(out, spec, Z, quant.K_ALPHA) for Z in (26, 29, 30)]
        sim.free_raw(out)
        sim.close()
        samples.append(quant.QuantSample(spec=spec, ilay=1, matrix=matrix, z_quant=[26, 29, 30], k_exp=k,
                                         l_exp=[0.0, 0.0, 0.0]))
    res = quant.quantify(samples, options=opts, gpu=gpu)
    for r, t in zip(res, truths):
        print("quantified", r.iterations, r.weights, "known", t)
        assert r.converged and r.iterations < quant.MAX_ITERATIONS
        assert r.sum_k <= quant.CONV_THRESHOLD
        np.testing.assert_allclose(r.weights, t, rtol=1e-2)
        assert sum(r.layer.weight) == pytest.approx(1.0)


def test_weight_update_rule_on_synthetic_histories():
    """One pass of the update of bin/xmimsim-pymca.c:652-770 on a made-up
    history: the K element grows by measured / simulated when that is below
    its jump limit, the L element is capped at its limit, and sum_k / sum_l
    are the squared relative misfits of the simulated intensities."""
    spec, matrix = _sample_spec([0.05, 0.03, 0.02], n=10)
    s = quant.QuantSample(spec=spec, ilay=1, matrix=Layer([8, 14], [0.5, 0.5], 2.5, 0.1), z_quant=[26, 82],
                          k_exp=[2.0, 0.0], l_exp=[0.0, 5.0], weights=[0.05, 0.005])
    st = quant._State(s)
    N = spec.n_interactions_trajectory
    vr = np.zeros((100, 385, N))
    lib = quant._xrl()
    kl2, kl3 = lib.xrl_line_from_name(b"KL2"), lib.xrl_line_from_name(b"KL3")
    l3m4, l3m5 = lib.xrl_line_from_name(b"L3M4"), lib.xrl_line_from_name(b"L3M5")
    vr[25, kl2 - 1, 0] = 0.5
    vr[25, kl3 - 1, 1] = 1.0
    vr[81, l3m4 - 1, 0] = 0.1
    vr[81, l3m5 - 1, 0] = 0.2
    st.update({"var_red": vr})
    k_sim = 0.5 * quant.detector_absorption(spec, 26, "KL2") + 1.0 * quant.detector_absorption(spec, 26, "KL3")
    l_sim = 0.1 * quant.detector_absorption(spec, 82, "L3M4") + 0.2 * quant.detector_absorption(spec, 82, "L3M5")
    assert st.k_sim[0] == pytest.approx(k_sim) and st.l_sim[1] == pytest.approx(l_sim)
    assert st.sum_k == pytest.approx(((2.0 - k_sim) / 2.0) ** 2)
    assert st.sum_l == pytest.approx(((5.0 - l_sim) / 5.0) ** 2)
    # Fe: 0.05 <= 0.1 -> limit 2.5; Pb: 0.005 <= 0.01 -> limit 10
    assert st.weights[0] == pytest.approx(0.05 * min(2.0 / k_sim, 2.5))
    assert st.weights[1] == pytest.approx(0.005 * min(5.0 / l_sim, 10.0))
    assert sum(st.layer.weight) == pytest.approx(1.0)


def test_unconverged_sample_stops_alone(monkeypatch):
    """A sample that cannot converge stops at max_iterations and comes back
    with converged = False while the other sample of the batch converges;
    strict=True raises instead.  The simulation is replaced by a stand-in that
    returns K-alpha histories proportional to the Fe weight (sample 0) or
    fixed (sample 1), so this runs on the CPU."""
    lib = quant._xrl()
    kl3 = lib.xrl_line_from_name(b"KL3")

    class FakeSim:
        def __init__(self, spec, options=None, gpu=None):
            self.spec = spec

        def solid_angle_grid(self):
            return {"r": None, "theta": None, "grid": None}

        def set_solid_angle(self, *a):
            pass

        @staticmethod
        def msim_batch(sims):
            outs = []
            for s in sims:
                lay = s.spec.layers[1]
                w_fe = lay.weight[lay.Z.index(26)]
                vr = np.zeros((100, 385, s.spec.n_interactions_trajectory))
                vr[25, kl3 - 1, 0] = 1e3 * w_fe if s.spec.live_time == 1.0 else 1e-3
                outs.append({"var_red": vr})
            return outs

        def free_raw(self, out):
            pass

        def close(self):
            pass

    monkeypatch.setattr(quant, "Simulation", FakeSim)
    samples = []
    for i in range(2):
        spec, matrix = _sample_spec([0.05, 0.03, 0.02], n=10)
        spec.live_time = 1.0 if i == 0 else 2.0  # marks the sample for the stand-in
        absorb = quant.detector_absorption(spec, 26, "KL3")
        samples.append(quant.QuantSample(spec=spec, ilay=1, matrix=matrix, z_quant=[26], k_exp=[50.0 * absorb],
                                         l_exp=[0.0]))
    res = quant.quantify(samples, options=dict(configs.C1_OPTIONS), max_iterations=12)
    assert res[0].converged and res[0].weights[0] == pytest.approx(0.05, rel=0.05)
    assert not res[1].converged and res[1].iterations == 12
    with pytest.raises(quant.XmiError):
        quant.quantify(samples, options=dict(configs.C1_OPTIONS), max_iterations=12, strict=True)
