"""GPU parity of the whole detector response (src/xmi_detector_f.F90:56-905)
against the FP64 oracle, called through the C-ABI
(xmi_detector_convolute_all) on the same tables and random streams:

* escape peaks (:582-809) with the escape-ratio tables the engine computes
  for the detector crystal (xmi_escape_ratios_calculation);
* pulse pile-up (:56-217) on the pulse-group Philox streams;
* Poisson noise (:862-905) on the per-channel Philox streams;
* all three together with the Gaussian + tail convolution, every order.

Tolerances: the convolved spectra at 1e-9 relative (the benchmark spec's bound is
1e-5: only the order of FP64 additions differs); the pile-up and Poisson
counts are integers drawn from identical streams and must be equal.
"""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

from xmimsim_gb300 import Simulation, configs, gpu_options

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
SEED = 0x5EED0001
PILE_SALT = 0x5055      # the engine's pile-up seed is gpu seed ^ this
POISSON_SALT = 0x9015   # and its Poisson seed gpu seed ^ this


def oracle():
    from oracle import oracle_api
    return oracle_api


def det_corr(spec):
    """Channel absorption factors of src/xmi_detector_f.F90:437-454 from the
    data model the engine tabulates with."""
    import xmimsim_gb300.tube as tube
    lib = tube._xrl()

    def layer_mu(l, E):
        w = np.array(l.weight) / sum(l.weight)
        return sum(wi * lib.xrl_CS_Total_Kissel(z, E) for z, wi in zip(l.Z, w))
    out = []
    for i in range(spec.nchannels):
        E = i * spec.gain + spec.zero
        d = 1.0
        for l in spec.det_layers:
            d *= math.exp(-l.density * l.thickness * layer_mu(l, E))
        for l in spec.crystal_layers:
            d = -d * math.expm1(-l.density * l.thickness * layer_mu(l, E))
        out.append(d)
    return np.array(out)


class EscapeTables:
    """The engine's escape-ratio tables and the oracle's view of them (same
    arrays; edges and line energies from the same data model)."""

    def __init__(self, sim, n_photons=20000, n_input_energies=200):
        import xmimsim_gb300.tube as tube
        xrl = tube._xrl()
        self.sim = sim
        self.ptr = sim.escape_ratios(n_photons=n_photons, n_input_energies=n_input_energies)
        er = self.ptr.contents
        nel, nfe = er.n_elements, er.n_fluo_input_energies
        nce, nco = er.n_compton_input_energies, er.n_compton_output_energies
        Z = [er.Z[i] for i in range(nel)]
        self.edge = np.array([[xrl.xrl_EdgeEnergy(z, sh) for sh in range(4)] for z in Z]).ravel()
        self.line_e = np.array([[xrl.xrl_LineEnergy(z, k) for k in range(1, 110)] for z in Z]).ravel()
        self.fluo = np.ctypeslib.as_array(er.fluo_escape_ratios, (nel * 109 * nfe,))
        self.comp = np.ctypeslib.as_array(er.compton_escape_ratios, (nce * nco,))
        dp = C.POINTER(C.c_double)
        self.oracle = oracle().OracleEscape(
            nel, nfe, nce, nco, self.edge.ctypes.data_as(dp), self.line_e.ctypes.data_as(dp),
            er.fluo_escape_ratios, er.fluo_escape_input_energies, er.compton_escape_ratios,
            er.compton_escape_input_energies, er.compton_escape_output_energies)

    def free(self):
        self.sim.lib.xmi_free_escape_ratios(self.ptr)


def oracle_chain(spec, noconv, dc, escape=None, pile=False, poisson=False):
    out = oracle().convolute_spectrum(noconv, dc, spec.gain, spec.zero, spec.fano, spec.noise, spec.detector_type,
                                      spec.live_time, spec.pulse_width, escape=escape,
                                      use_sum_peaks=1 if pile else 0, pile_seed=SEED ^ PILE_SALT)
    if poisson:
        out = oracle().poisson(out, SEED ^ POISSON_SALT)
    return out


@pytest.fixture(scope="module")
def c1_run():
    """A C1 spectrum (20000 photons, every order) and the engine's escape
    tables of its Si crystal."""
    spec = configs.config1(n_photons_line=20000)
    spec.live_time = 60.0  # a count rate whose 10 us pulses pile up in small groups
    sim = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))
    sim.solid_angle()
    out = sim.msim()
    esc = EscapeTables(sim)
    yield spec, sim, out["channels"], esc
    esc.free()
    sim.free_raw(out)
    sim.close()


def test_escape_peaks_match_oracle(c1_run):
    spec, sim, channels, esc = c1_run
    sim.options.use_escape_peaks, sim.options.use_sum_peaks, sim.options.use_poisson = 1, 0, 0
    conv = sim.convolute(channels, escape=esc.ptr)
    dc = det_corr(spec)
    moved = 0.0
    for k in range(1, spec.n_interactions_trajectory + 1):
        ref = oracle_chain(spec, channels[k], dc, escape=esc.oracle)
        np.testing.assert_allclose(conv[k], ref, rtol=1e-9, atol=1e-12 * ref.max(), err_msg="order %d" % k)
        plain = oracle_chain(spec, channels[k], dc)
        moved = max(moved, np.abs(ref - plain).max() / ref.max())
    # the escape tables must actually move counts (Si K escape, Compton escape)
    assert moved > 1e-4


def test_escape_step_alone_matches_oracle(c1_run):
    """The escape step on a spectrum with counts in every channel (a gamma
    continuum plus eight strong peaks), so that every channel's Compton and
    fluorescence escape transfer contributes."""
    spec, sim, channels, esc = c1_run
    rng = np.random.default_rng(11)
    x = rng.gamma(2.0, 100.0, size=spec.nchannels)
    x[rng.choice(spec.nchannels, 8, replace=False)] += 1e6
    noconv = np.zeros((2, spec.nchannels))
    noconv[1] = x
    sim.options.use_escape_peaks, sim.options.use_sum_peaks, sim.options.use_poisson = 1, 0, 0
    conv = sim.convolute(noconv, escape=esc.ptr)[1]
    ref = oracle_chain(spec, x, det_corr(spec), escape=esc.oracle)
    np.testing.assert_allclose(conv, ref, rtol=1e-9, atol=1e-12 * ref.max())


def test_pile_up_matches_oracle_srm1155():
    """The pulse train of tests/test-pile-up.c's spectrum (srm1155, 5.8e6
    pulses over 300 s, pulse width 0.203 us) on the same pulse-group streams:
    the piled-up spectrum is the oracle's, count for count (the convolved
    spectra agree to the order of FP64 additions), and channel 1077 gains
    more than a hundredfold as the reference test requires."""
    from xmimsim_gb300 import xmlio
    g = json.loads((GOLDEN / "srm1155.json").read_text())
    spec = xmlio.read_xmsi(g["xmsi"])
    spec.n_photons_line = spec.n_photons_interval = 1
    sim = Simulation(spec, options=dict(use_escape_peaks=0, use_sum_peaks=1, use_default_seeds=1),
                     gpu=gpu_options(seed=SEED))
    unconv = np.zeros((spec.n_interactions_trajectory + 1, spec.nchannels))
    unconv[-1] = g["unconv_last"]
    conv = sim.convolute(unconv)[-1]
    dc = det_corr(spec)
    ref = oracle_chain(spec, unconv[-1], dc, pile=True)
    np.testing.assert_allclose(conv, ref, rtol=1e-9, atol=1e-12 * ref.max())
    # the pile-up step alone, before convolution: integer counts, conserved pulses
    piled = oracle().sum_peaks(unconv[-1] * dc, spec.live_time, spec.pulse_width, spec.gain, spec.zero,
                               SEED ^ PILE_SALT)
    assert np.array_equal(piled, np.round(piled))
    assert piled.sum() < (unconv[-1] * dc).sum()
    sim.options.use_sum_peaks = 0
    without = sim.convolute(unconv)[-1]
    assert conv[g["pileup_channel"]] / without[g["pileup_channel"]] > g["pileup_min_ratio"]
    sim.close()


def test_poisson_matches_oracle(c1_run):
    """Poisson noise on the convolved spectrum: channel i's variate comes from
    the Philox stream (seed, i, 0xE0000000), so the engine's counts equal the
    oracle's (exact multiplication / PTRS draws on both sides)."""
    spec, sim, channels, esc = c1_run
    sim.options.use_escape_peaks, sim.options.use_sum_peaks, sim.options.use_poisson = 0, 0, 1
    scaled = channels * (1e5 / channels[1:].max())  # means from below 1 to 1e5 counts per channel
    conv = sim.convolute(scaled)
    dc = det_corr(spec)
    n_drawn = 0
    for k in range(1, spec.n_interactions_trajectory + 1):
        ref = oracle_chain(spec, scaled[k], dc, poisson=True)
        mean = oracle_chain(spec, scaled[k], dc)
        drawn = mean > 1.0
        n_drawn += int(drawn.sum())
        assert np.array_equal(conv[k][drawn], np.round(conv[k][drawn]))
        # channels at or below one count are left as they are
        np.testing.assert_allclose(conv[k][~drawn], mean[~drawn], rtol=1e-9, atol=1e-300)
        assert (conv[k][drawn] == ref[drawn]).mean() >= 0.999, "order %d" % k
    assert n_drawn > 1000
    sim.options.use_poisson = 0


def test_poisson_is_poisson(c1_run):
    """Size-independent property of the engine's Poisson step: over every
    drawn channel of several spectra, (k - lam)/sqrt(lam) has mean 0 and
    variance 1, and for small means the counts' skewness is 1/sqrt(lam)."""
    spec, sim, channels, esc = c1_run
    sim.options.use_escape_peaks, sim.options.use_sum_peaks = 0, 0
    z_all, small = [], []
    for top in (10.0, 30.0, 100.0, 300.0, 3e3, 3e4, 3e5):
        x = channels * (top / channels[1:].max())
        sim.options.use_poisson = 0
        lam = sim.convolute(x)
        sim.options.use_poisson = 1
        k = sim.convolute(x)
        m = lam > 1.0
        z_all.append(((k - lam) / np.sqrt(np.where(m, lam, 1.0)))[m])
        s = m & (lam < 20.0)
        ls = np.where(s, lam, 1.0)
        small.append(((k - lam) ** 3 / ls ** 1.5 - 1.0 / np.sqrt(ls))[s])
    z = np.concatenate(z_all)
    n = len(z)
    assert n > 8000
    assert abs(z.mean()) < 5.0 / math.sqrt(n)
    assert abs(z.var() - 1.0) < 6.0 * math.sqrt(2.0 / n)
    sk = np.concatenate(small)
    assert len(sk) > 200
    assert abs(sk.mean()) < 6.0 * sk.std() / math.sqrt(len(sk))
    sim.options.use_poisson = 0


def test_full_detector_response_matches_oracle(c1_run):
    """Escape peaks, pile-up, convolution and Poisson noise together, every
    order of C1, through xmi_detector_convolute_all; the spectrum is scaled
    to 3e6 pulses in the first order over the 60 s live time (0.5 pulses per
    10 us pulse width)."""
    spec, sim, channels, esc = c1_run
    sim.options.use_escape_peaks, sim.options.use_sum_peaks, sim.options.use_poisson = 1, 1, 1
    dc = det_corr(spec)
    scale = 3e6 / max((channels[1] * dc).sum(), 1e-300)
    x = channels * scale
    conv = sim.convolute(x, escape=esc.ptr)
    for k in range(1, spec.n_interactions_trajectory + 1):
        ref = oracle_chain(spec, x[k], dc, escape=esc.oracle, pile=True, poisson=True)
        drawn = ref > 1.0
        assert (conv[k][drawn] == ref[drawn]).mean() >= 0.999, "order %d" % k
        np.testing.assert_allclose(conv[k].sum(), ref.sum(), rtol=1e-4)
    sim.options.use_escape_peaks, sim.options.use_sum_peaks, sim.options.use_poisson = 1, 0, 0
