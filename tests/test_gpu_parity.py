"""GPU parity: the CUDA engine, called through its C-ABI, against the FP64 CPU
oracle on the same tables, Philox streams and solid-angle grid.

Tolerances: FP64 transport and grids are compared at rtol 1e-6 (identical
random sequences and arithmetic up to FMA contraction / last-ulp differences of
the math libraries; a rare channel-boundary flip moves one contribution to a
neighbouring channel, hence the channel check on sums and at 1e-4 per
channel); the FP32 transport consumes the same draws and is compared at 2e-3
on the main line intensities; the detector convolution at 1e-9.
"""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

from xmimsim_gb300 import DiscreteLine, ContinuousPoint, InputSpec, Layer, Simulation, configs, gpu_options

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
SEED = 0x5EED0001


def oracle():
    from oracle import oracle_api
    return oracle_api


def run_pair(spec, options, precision=0, hits=None):
    sim = Simulation(spec, options=options, gpu=gpu_options(precision=precision, seed=SEED))
    if options.get("use_variance_reduction", 1):
        sim.solid_angle()
    gpu = sim.msim()
    sim.prepare()
    ref = oracle().msim(sim.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels)
    return sim, gpu, ref


def assert_transport_equal(gpu, ref, rtol=1e-6):
    for key in ("var_red", "brute"):
        g, o = gpu[key], ref[key]
        if g is None:
            assert not o.any()
            continue
        scale = max(abs(o).max(), 1e-300)
        np.testing.assert_allclose(g, o, rtol=rtol, atol=rtol * scale * 1e-3)
    cg, co = gpu["channels"], ref["channels"]
    np.testing.assert_allclose(cg.sum(axis=1), co.sum(axis=1), rtol=rtol)
    np.testing.assert_allclose(cg, co, rtol=1e-4, atol=1e-4 * max(co.max(), 1e-300))


def test_solid_angle_grid_matches_oracle_exactly():
    spec = configs.config1(n_photons_line=10)
    sim = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))
    g = sim.solid_angle_grid()
    sim.prepare()
    nr, nt = len(g["r"]), len(g["theta"])
    rng = np.random.default_rng(1)
    pts = np.sort(rng.choice(nr * nt, size=256, replace=False))
    vals = np.array([oracle().solid_angle_points(sim.bundle_ptr(), g["r"], g["theta"], int(p), int(p) + 1, 5000)[0]
                     for p in pts])
    gpu_vals = g["grid"].reshape(-1)[pts]
    # identical hit counts: equal values; allow a single boundary flip on a handful of points
    diff = np.abs(gpu_vals - vals)
    quantum = np.maximum(vals, gpu_vals) / 5000.0 * 1.5 + 1e-300
    assert (diff <= quantum).all()
    assert (diff == 0).mean() > 0.95
    sim.close()


@pytest.mark.parametrize("precision", [1, 0])
@pytest.mark.parametrize("name", ["no_collimator", "conical_collimator", "conical_collimator_wide"])
def test_solid_angle_grid_matches_reference_opencl_kernel(name, precision):
    """The GPU grid drawn from the OpenCL kernel's own Threefry stream against
    that kernel's results at 600 points per geometry (src/xmi_kernels.cl run
    on the host, tests/golden/cl_solid_angle.json).  The reference evaluates
    in FP32 with the host's math library, the GPU with CUDA's, so a sample on
    the detector or aperture rim can fall either way: hit counts agree exactly
    at most points and within a few hits everywhere, without bias.  FP64 also
    agrees with the FP64 oracle on the same stream."""
    import test_oracle as T
    g = json.loads((GOLDEN / "cl_solid_angle.json").read_text())
    d = g["geometries"][name]
    sim = Simulation(T.cl_geometries()[name], options=dict(use_variance_reduction=1, use_escape_peaks=0,
                                                           use_default_seeds=1),
                     gpu=gpu_options(precision=precision, seed=SEED, solid_angle_stream=1))
    grid = sim.solid_angle_grid()
    vals = grid["grid"][d["it"], d["ir"]]
    hg = T.hits_of(vals, d["cone_solid_angle"], g["hits_per_single"])
    hr = T.hits_of(d["value"], d["cone_solid_angle"], g["hits_per_single"])
    dh = hg - hr
    assert (dh == 0).mean() > 0.85
    assert np.abs(dh).max() <= 5
    assert abs(dh.sum()) <= 4.0 * math.sqrt(max(1.0, (dh ** 2).sum()))
    if precision == 0:
        sim.prepare()
        o = oracle().solid_angle_points_cl_stream(sim.bundle_ptr(), grid["r"], grid["theta"], d["ir"], d["it"],
                                                  g["hits_per_single"])
        ho = T.hits_of(o, d["cone_solid_angle"], g["hits_per_single"])
        assert (hg == ho).mean() > 0.99
    sim.close()


def test_solid_angle_grid_fp32_close_to_fp64():
    spec = configs.config1(n_photons_line=10)
    s64 = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))
    s32 = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(precision=1, seed=SEED))
    g64, g32 = s64.solid_angle_grid()["grid"], s32.solid_angle_grid()["grid"]
    m = g64 > 1e-4
    assert np.median(np.abs(g32[m] - g64[m]) / g64[m]) < 1e-3
    s64.close()
    s32.close()


def test_transport_fp64_config1_matches_oracle():
    spec = configs.config1(n_photons_line=20000)
    sim, gpu, ref = run_pair(spec, configs.C1_OPTIONS)
    assert_transport_equal(gpu, ref)
    assert gpu["var_red"][26 - 1, 3 - 1].sum() > 0  # Fe-KL3
    sim.close()


def mixed_source_spec():
    layers = configs.random_layers(seed=11, n_layers=3, nel=(2, 5), thick=(1e-4, 0.05))
    cont = [ContinuousPoint(5.0 + i, 1e8 * (1 + 0.1 * i), 5e7) for i in range(12)]
    disc = [DiscreteLine(16.0, 1e9, 1e8, distribution_type=1, scale_parameter=0.05),
            DiscreteLine(12.0, 5e8, 5e8, distribution_type=2, scale_parameter=0.02),
            DiscreteLine(9.0, 1e9, 0.0, sigma_x=0.01, sigma_xp=0.001, sigma_y=0.01, sigma_yp=0.001)]
    return InputSpec(layers=layers, reference_layer=2, n_photons_interval=300, n_photons_line=1500,
                     n_interactions_trajectory=5, p_detector_window=(0.0, 10.0, 100.0), discrete=disc,
                     continuous=cont, exc_layers=[Layer([13], [1.0], 2.7, 0.01)])


def test_transport_fp64_mixed_sources_multilayer_matches_oracle():
    spec = mixed_source_spec()
    sim, gpu, ref = run_pair(spec, dict(configs.C1_OPTIONS))
    assert_transport_equal(gpu, ref)
    sim.close()


@pytest.mark.parametrize("cascade", [(0, 0), (1, 0), (0, 1)])
def test_transport_cascade_options_match_oracle(cascade):
    spec = configs.config1(n_photons_line=5000)
    opts = dict(configs.C1_OPTIONS, use_cascade_auger=cascade[0], use_cascade_radiative=cascade[1], use_M_lines=0)
    sim, gpu, ref = run_pair(spec, opts)
    assert_transport_equal(gpu, ref)
    sim.close()


def test_transport_analog_brute_force_matches_oracle():
    spec = configs.config1(n_photons_line=200000)
    spec.p_detector_window = (0.0, 1.0, 100.0)
    opts = dict(configs.C1_OPTIONS, use_variance_reduction=0)
    sim, gpu, ref = run_pair(spec, opts)
    assert gpu["var_red"] is None
    assert_transport_equal(gpu, ref)
    sim.close()


def collimator_spec(n=5000):
    spec = configs.config1(n_photons_line=n)
    spec.collimator_height = 1.0
    spec.collimator_diameter = 0.2
    return spec


def test_transport_collimator_matches_oracle():
    sim, gpu, ref = run_pair(collimator_spec(), configs.C1_OPTIONS)
    assert_transport_equal(gpu, ref)
    sim.close()


def test_transport_fp32_tracks_fp64():
    spec = configs.config1(n_photons_line=50000)
    s64 = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(precision=0, seed=SEED))
    s32 = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(precision=1, seed=SEED))
    r64, r32 = s64.msim(), s32.msim()
    for Z, line in ((26, 3), (29, 3), (30, 3), (26, 2), (29, 6)):
        a, b = r64["var_red"][Z - 1, line - 1].sum(), r32["var_red"][Z - 1, line - 1].sum()
        assert b == pytest.approx(a, rel=2e-3)
    np.testing.assert_allclose(r32["channels"].sum(axis=1), r64["channels"].sum(axis=1), rtol=2e-3)
    s64.close()
    s32.close()


def test_invalid_input_fails_cleanly():
    from xmimsim_gb300 import XmiError
    spec = configs.config1(n_photons_line=10)
    spec.n_interactions_trajectory = 99
    with pytest.raises(XmiError):
        Simulation(spec, options=configs.C1_OPTIONS)


def test_detector_convolution_matches_oracle():
    spec = configs.config1(n_photons_line=20000)
    sim = Simulation(spec, options=dict(configs.C1_OPTIONS, use_escape_peaks=0), gpu=gpu_options(seed=SEED))
    out = sim.msim()
    conv = sim.convolute(out["channels"])
    # channel absorption factors the engine applies, recomputed with the data model
    import xmimsim_gb300.tube as tube
    lib = tube._xrl()

    def layer_mu(l, E):
        w = np.array(l.weight) / sum(l.weight)
        return sum(wi * lib.xrl_CS_Total_Kissel(z, E) for z, wi in zip(l.Z, w))
    dc = []
    for i in range(spec.nchannels):
        E = i * spec.gain + spec.zero
        d = 1.0
        for l in spec.det_layers:
            d *= math.exp(-l.density * l.thickness * layer_mu(l, E))
        for l in spec.crystal_layers:
            d = -d * math.expm1(-l.density * l.thickness * layer_mu(l, E))
        dc.append(d)
    for k in range(1, spec.n_interactions_trajectory + 1):
        ref = oracle().convolute_spectrum(out["channels"][k], np.array(dc), spec.gain, spec.zero, spec.fano,
                                          spec.noise, spec.detector_type, spec.live_time, spec.pulse_width)
        np.testing.assert_allclose(conv[k], ref, rtol=1e-9, atol=1e-12 * ref.max())
    sim.close()


def test_pile_up_reference_srm1155():
    """tests/test-pile-up.c: with pile-up the counts at channel 1077 of the
    srm1155 example rise more than a hundredfold."""
    from xmimsim_gb300 import xmlio
    g = json.loads((GOLDEN / "srm1155.json").read_text())
    spec = xmlio.read_xmsi(g["xmsi"])
    spec.n_photons_line = spec.n_photons_interval = 1
    sim = Simulation(spec, options=dict(use_escape_peaks=0, use_sum_peaks=0, use_default_seeds=1))
    unconv = np.zeros((spec.n_interactions_trajectory + 1, spec.nchannels))
    unconv[-1] = g["unconv_last"]
    without = sim.convolute(unconv)[-1][g["pileup_channel"]]
    sim.options.use_sum_peaks = 1
    with_pu = sim.convolute(unconv)[-1][g["pileup_channel"]]
    assert with_pu / without > g["pileup_min_ratio"]
    sim.close()


def test_escape_ratios_plausible():
    spec = configs.config1(n_photons_line=10)
    sim = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))
    er = sim.escape_ratios(n_photons=20000, n_input_energies=100).contents
    nel, nE = er.n_elements, er.n_fluo_input_energies
    fluo = np.ctypeslib.as_array(er.fluo_escape_ratios, (nE * 109 * nel,)).reshape(nE, 109, nel)
    E = np.ctypeslib.as_array(er.fluo_escape_input_energies, (nE,))
    si_k = fluo[:, 2, 0] + fluo[:, 1, 0]  # Si KL3 + KL2
    above = E > 2.0
    assert (si_k[above] > 0).all() and (si_k[above] < 0.2).all()
    assert (si_k[E < 1.8] == 0).all()
    sim.lib.xmi_free_escape_ratios(C.pointer(er))
    sim.close()


def test_batched_run_matches_single_runs_and_oracle():
    """xmi_main_msim_batch: three different configurations in one launch
    sequence give each configuration's single-run result (same photon
    streams; only the order of FP64 additions differs) and the oracle's."""
    specs = [configs.config1(n_photons_line=4000), mixed_source_spec(), collimator_spec(3000)]
    specs[0].n_interactions_trajectory = 3
    sims = [Simulation(sp, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED)) for sp in specs]
    for s in sims:
        s.solid_angle()
    batched = Simulation.msim_batch(sims)
    for s, b in zip(sims, batched):
        single = s.msim()
        np.testing.assert_allclose(b["var_red"], single["var_red"], rtol=1e-9, atol=1e-12 * abs(single["var_red"]).max())
        np.testing.assert_allclose(b["channels"], single["channels"], rtol=1e-9,
                                   atol=1e-12 * abs(single["channels"]).max())
        s.prepare()
        ref = oracle().msim(s.bundle_ptr(), s.spec.n_interactions_trajectory, s.spec.nchannels)
        assert_transport_equal(b, ref)
        s.free_raw(b)
        s.free_raw(single)
        s.close()


def test_transport_fp32_tracks_fp64_production_stack():
    """FP32 transport on the 5-layer Rh-tube stack (the production workload at
    a small budget) against the FP64 run on the same photon streams: total
    estimator tally within 1e-3, the 20 strongest lines within 1e-2, and no
    point of the solid-angle grid is missed (the off-grid Monte Carlo count
    matches FP64's)."""
    spec = configs.config2(total_photons=200000)
    opts = dict(configs.C2_OPTIONS, use_sum_peaks=0)
    s64 = Simulation(spec, options=opts, gpu=gpu_options(precision=0, seed=SEED))
    s32 = Simulation(spec, options=opts, gpu=gpu_options(precision=1, seed=SEED))
    r64, r32 = s64.msim(), s32.msim()
    v64, v32 = r64["var_red"].sum(axis=2), r32["var_red"].sum(axis=2)
    assert v32.sum() == pytest.approx(v64.sum(), rel=1e-3)
    top = np.argsort(v64.ravel())[-20:]
    np.testing.assert_allclose(v32.ravel()[top], v64.ravel()[top], rtol=1e-2)
    s64.close()
    s32.close()


def test_autotuned_batch_keeps_results():
    """xmi_gpu_autotune_batch picks a launch shape and queue size from its
    candidates, writes them into every configuration, and the batched run with
    them gives the untuned run's result (photon streams are keyed by photon,
    not by launch shape; only the order of FP64 additions differs)."""
    specs = [configs.config1(n_photons_line=3000), mixed_source_spec()]
    sims = [Simulation(sp, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED)) for sp in specs]
    before = Simulation.msim_batch(sims)
    tune = Simulation.autotune_batch(sims, share=0.5)
    assert tune["threads_per_block"] in (64, 128) and tune["blocks_per_sm"] in (4, 8, 12, 16)
    assert tune["queue_events"] in (1 << 23, 1 << 24, 1 << 25) and tune["best_trial_ms"] > 0
    after = Simulation.msim_batch(sims)
    for s, a, b in zip(sims, before, after):
        assert s.gpu.blocks_per_sm == tune["blocks_per_sm"]
        np.testing.assert_allclose(b["var_red"], a["var_red"], rtol=1e-9, atol=1e-12 * abs(a["var_red"]).max())
        s.free_raw(a)
        s.free_raw(b)
        s.close()


def test_batched_graph_is_updated_in_place():
    """The second batched call of the same configurations reuses the first
    call's executable graph (cudaGraphExecUpdate with the new call's buffers
    and events) and gives the same result; a batch of another shape gets a
    graph of its own."""
    from xmimsim_gb300 import last_timing
    specs = [configs.config1(n_photons_line=3000), mixed_source_spec()]
    sims = [Simulation(sp, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED)) for sp in specs]
    first = Simulation.msim_batch(sims)
    second = Simulation.msim_batch(sims)
    assert last_timing()["graph_updated"] == 1
    for s, a, b in zip(sims, first, second):
        np.testing.assert_allclose(b["var_red"], a["var_red"], rtol=1e-9, atol=1e-12 * abs(a["var_red"]).max())
        np.testing.assert_allclose(b["channels"], a["channels"], rtol=1e-9, atol=1e-12 * abs(a["channels"]).max())
        s.free_raw(a)
        s.free_raw(b)
    one = Simulation.msim_batch(sims[:1])
    # another shape: the update is refused (100 + cudaGraphExecUpdateErrorTopologyChanged) and a new graph runs
    assert last_timing()["graph_updated"] >= 100
    np.testing.assert_allclose(one[0]["var_red"], second[0]["var_red"], rtol=1e-9,
                               atol=1e-12 * abs(second[0]["var_red"]).max())
    sims[0].free_raw(one[0])
    for s in sims:
        s.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_overlapped_chunks_match_serial(precision):
    """With variance reduction and several chunks, chunk k+1's transport runs
    beside chunk k's sort, solid angles and estimator (second stream, two
    event queues).  Histories and spectra equal those of the chunks run one
    after another, through the single-configuration call and the batched
    graph; FP64 to the order of its atomics, FP32 to the rounding of its
    per-warp partial sums (the counting sort's order within a key varies)."""
    from xmimsim_gb300 import last_timing
    specs = [configs.config1(n_photons_line=40000), mixed_source_spec()]
    rtol = 1e-9 if precision == 0 else 2e-5
    sims = [Simulation(sp, options=configs.C1_OPTIONS, gpu=gpu_options(precision=precision, seed=SEED))
            for sp in specs]
    runs = {}
    for serial in (1, 0):
        g = gpu_options(precision=precision, seed=SEED, overlap_chunks=1 - serial)
        g.queue_events = 1 << 16  # 2^16 / 4 interactions: 16384 photons per chunk
        for sim in sims:
            sim.set_gpu(g)
        single = sims[0].msim()
        t_single = last_timing()
        batch = Simulation.msim_batch(sims)
        t_batch = last_timing()
        runs[serial] = (single, t_single, batch, t_batch)
    (one1, t1, b1, tb1), (one0, t0, b0, tb0) = runs[1], runs[0]
    assert t0["events"] == t1["events"] > 0 and tb0["events"] == tb1["events"] > 0
    assert t0["launches"] == t1["launches"] > 40  # several chunks
    for a, b in [(one1, one0)] + list(zip(b1, b0)):
        for key in ("var_red", "channels"):
            np.testing.assert_allclose(b[key], a[key], rtol=rtol, atol=rtol * abs(a[key]).max())
    for single, _, batch, _ in runs.values():
        sims[0].free_raw(single)
        for s, o in zip(sims, batch):
            s.free_raw(o)
    for s in sims:
        s.close()


def test_surrogate_integrator_fallback_matches_oracle():
    """Estimator events outside the network's checked region go to the
    warp-parallel integrator (omega_fallback_kernel), which must reproduce the
    serial off-grid integral of the grid path draw for draw.  A network
    trained on points far from the sample leaves every event outside; the
    oracle, given a grid whose r axis ends below every event's distance (so
    every event is off-grid), computes the same integrals on the same
    streams: the two transports agree."""
    spec = configs.config1(n_photons_line=3000)
    sur = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED, use_surrogate=1))
    rng = np.random.default_rng(7)
    n = (1 << 14) + 4096
    sur.build_surrogate_points(rng.uniform(50.0, 60.0, n), rng.uniform(0.5, 1.0, n), hits_train=64, epochs=1,
                               hits_check=1 << 8)
    out = sur.msim()
    tm = sur.timing()
    assert tm["surrogate_fallbacks"] == tm["events"] > 0
    ref = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))
    r, t = ref.grid_axes(16, 16)
    ref.set_solid_angle(np.linspace(1e-3, 1e-2, 16), t, np.zeros((16, 16)))
    ref.prepare()
    o = oracle().msim(ref.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels)
    assert o["not_found"] > 0
    assert_transport_equal(out, o)
    sur.free_raw(out)
    sur.close()
    ref.close()


def test_thin_layers_fp32_tracks_fp64():
    """Config 3, the precision form of config 1 (10 nm Cr and 50 nm Au over a
    2 mm substrate): FP32 transport with FP64 plane heights against the
    all-FP64 run on the same photon streams -- every line carrying >= 1% of
    the strongest within 0.5%, the thin layers' own lines (Cr K, Au L)
    included, and the channel totals within 0.5%."""
    spec = configs.config3(n_photons_line=200000)
    s64 = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(precision=0, seed=SEED))
    s32 = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(precision=1, seed=SEED))
    r64, r32 = s64.msim(), s32.msim()
    v64, v32 = r64["var_red"].sum(axis=2), r32["var_red"].sum(axis=2)
    assert v64[24 - 1, 3 - 1] > 0 and v64[79 - 1].sum() > 0  # Cr KL3 and Au L lines exist
    big = v64 > 1e-2 * v64.max()
    rel = np.abs(v32[big] - v64[big]) / v64[big]
    assert rel.max() < 5e-3, (rel.max(), np.argwhere(big)[rel.argmax()])
    for Z, line in ((24, 3), (79, 3 + 0)):
        if v64[Z - 1, line - 1] > 1e-3 * v64.max():
            assert v32[Z - 1, line - 1] == pytest.approx(v64[Z - 1, line - 1], rel=5e-3)
    np.testing.assert_allclose(r32["channels"].sum(axis=1), r64["channels"].sum(axis=1), rtol=5e-3)
    s64.close()
    s32.close()


def test_escape_ratios_match_oracle():
    """Escape ratios (src/xmi_main.F90:5473-5800): the GPU escape-mode Monte
    Carlo against the FP64 oracle on the same escape tables and Philox
    streams -- fluorescence and Compton escape ratios equal to within the
    order of FP64 additions, for input energies across the Si K edge."""
    from xmimsim_gb300 import abi
    spec = configs.config1(n_photons_line=10)
    sim = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))
    nE, n_ph = 40, 4000
    er = sim.escape_ratios(n_photons=n_ph, n_input_energies=nE).contents
    nel, nco = er.n_elements, er.n_compton_output_energies
    fluo_g = np.ctypeslib.as_array(er.fluo_escape_ratios, (nE * 109 * nel,)).reshape(nE, 109, nel)
    comp_g = np.ctypeslib.as_array(er.compton_escape_ratios, (nco * nE,)).reshape(nco, nE)
    E = np.ctypeslib.as_array(er.fluo_escape_input_energies, (nE,)).copy()
    co = np.ctypeslib.as_array(er.compton_escape_output_energies, (nco,)).copy()
    lib = abi.load()
    h, t = C.c_void_p(), C.c_void_p()
    assert lib.xmi_gpu_escape_tables(C.byref(sim.cinput.input), C.byref(sim.options), C.byref(h), C.byref(t)) == 1
    f, c, it = oracle().escape_ratios(lib.xmi_gpu_bundle(t), nel, nE, E[0], E[1] - E[0], n_ph, nco, co[0],
                                      co[1] - co[0])
    assert (it > 0).all()
    fluo_o = f / it[:, None, None]          # [nE][nel][109]
    comp_o = c / it[:, None]                 # [nE][nco]
    np.testing.assert_allclose(fluo_g.transpose(0, 2, 1), fluo_o, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(comp_g.T, comp_o, rtol=1e-9, atol=1e-12)
    assert fluo_o[E > 2.0].sum() > 0        # Si K escape above the edge
    lib.xmi_free_hdf5_F(C.byref(t))
    lib.xmi_free_input_F(C.byref(h))
    sim.lib.xmi_free_escape_ratios(C.pointer(er))
    sim.close()


def heavy_layer_spec(n=5000):
    spec = configs.config1(n_photons_line=n)
    spec.layers = [Layer([82, 8, 26], [0.6, 0.3, 0.1], 5.0, 0.01)]
    spec.reference_layer = 1
    return spec


@pytest.mark.parametrize("which", ["config1", "mixed", "lead"])
def test_advanced_compton_fp64_matches_oracle(which):
    """use_advanced_compton = 1: the per-shell impulse-approximation Compton
    scattering of the transport (src/xmi_main.F90:4785-4983) and of the
    estimator (src/xmi_variance_reduction.F90:752-947), FP64 GPU against the
    oracle on the same profile tables and photon streams."""
    spec = {"config1": lambda: configs.config1(n_photons_line=20000), "mixed": mixed_source_spec,
            "lead": heavy_layer_spec}[which]()
    sim, gpu, ref = run_pair(spec, dict(configs.C1_OPTIONS, use_advanced_compton=1))
    assert_transport_equal(gpu, ref)
    assert gpu["var_red"][:, 384].sum() > 0
    sim.close()


def test_advanced_compton_fp32_and_batched():
    """FP32 transport with the advanced Compton scattering tracks FP64 (2e-3
    on the line totals and the spectrum orders), and a batch mixing an
    advanced-Compton configuration with a default one gives each its single
    run's result."""
    spec = heavy_layer_spec(20000)
    opts = dict(configs.C1_OPTIONS, use_advanced_compton=1)
    s64 = Simulation(spec, options=opts, gpu=gpu_options(precision=0, seed=SEED))
    s32 = Simulation(spec, options=opts, gpu=gpu_options(precision=1, seed=SEED))
    r64, r32 = s64.msim(), s32.msim()
    v64, v32 = r64["var_red"].sum(axis=2), r32["var_red"].sum(axis=2)
    assert v32.sum() == pytest.approx(v64.sum(), rel=2e-3)
    assert v32[:, 384].sum() == pytest.approx(v64[:, 384].sum(), rel=2e-3)
    np.testing.assert_allclose(r32["channels"].sum(axis=1), r64["channels"].sum(axis=1), rtol=2e-3)
    # the shape of the first-order Compton peak (15.5-17.2 keV: the 17.44 keV
    # beam scattered near 90 degrees, Doppler-broadened; Rayleigh and lines
    # outside), channel by channel: FP32 and FP64 draw the same shells and
    # momenta, so only channel-boundary flips of the scattered energy differ
    lo, hi = int(15.5 / spec.gain), int(17.2 / spec.gain)
    w64, w32 = r64["channels"][1][lo:hi], r32["channels"][1][lo:hi]
    big = w64 > 0.05 * w64.max()
    assert big.sum() > 20
    np.testing.assert_allclose(w32[big], w64[big], rtol=1e-2)
    x = np.arange(lo, hi)
    c64, c32 = (x * w64).sum() / w64.sum(), (x * w32).sum() / w32.sum()
    assert abs(c32 - c64) < 0.05  # centroid within 1/20 of a channel
    sd64 = math.sqrt(((x - c64) ** 2 * w64).sum() / w64.sum())
    sd32 = math.sqrt(((x - c32) ** 2 * w32).sum() / w32.sum())
    assert sd32 == pytest.approx(sd64, rel=2e-3)
    s64.close()
    s32.close()
    sims = [Simulation(heavy_layer_spec(3000), options=opts, gpu=gpu_options(seed=SEED)),
            Simulation(mixed_source_spec(), options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))]
    for s in sims:
        s.solid_angle()
    batched = Simulation.msim_batch(sims)
    for s, b in zip(sims, batched):
        single = s.msim()
        np.testing.assert_allclose(b["var_red"], single["var_red"], rtol=1e-9,
                                   atol=1e-12 * abs(single["var_red"]).max())
        np.testing.assert_allclose(b["channels"], single["channels"], rtol=1e-9,
                                   atol=1e-12 * abs(single["channels"]).max())
        s.free_raw(b)
        s.free_raw(single)
        s.close()


def test_compton_kinematics_fp32_sweep():
    """The FP32 kinematics of the advanced Compton path on the GPU against the
    FP64 formulas of the reference (oracle), evaluated at the same
    FP32-rounded inputs, over photon energies 1-150 keV, binding energies
    0-5 keV, angles from 1e-3 rad to pi and Q of both signs:
    * the scattered energy E(Q) (the cancellation-free quadratic, both roots)
      within 2e-6 relative, median below 3e-7;
    * Qimax (the half-angle form) within 2e-6 of its scale, down to small
      angles where the reference form loses digits in FP32;
    * the FP64 device functions equal the oracle's to 1e-8."""
    from xmimsim_gb300 import abi
    lib = abi.load()
    rng = np.random.default_rng(3)
    n = 40000
    E = np.exp(rng.uniform(np.log(1.0), np.log(150.0), n))
    Ii = np.where(rng.uniform(size=n) < 0.2, 0.0, rng.uniform(0.0, 1.0, n) * np.minimum(5.0, 0.9 * E))
    th = np.where(rng.uniform(size=n) < 0.3, np.exp(rng.uniform(np.log(1e-3), np.log(0.1), n)),
                  rng.uniform(0.1, math.pi, n))
    Q = rng.choice([-1.0, 1.0], n) * np.exp(rng.uniform(np.log(0.01), np.log(99.0), n))
    E, Ii, th, Q = (np.ascontiguousarray(v.astype(np.float32).astype(np.float64)) for v in (E, Ii, th, Q))
    out = np.zeros((n, 6))
    dp = abi.c_double_p
    assert lib.xmi_gpu_compton_kinematics(n, E.ctypes.data_as(dp), Ii.ctypes.data_as(dp), th.ctypes.data_as(dp),
                                          Q.ctypes.data_as(dp), out.ctypes.data_as(dp)) == 1, abi.last_error()
    q32, q64, e32, e64, bad32, bad64 = out.T
    ref_q = np.array([oracle().compton_qimax(a, b, c) for a, b, c in zip(E, Ii, th)])
    ref_e = np.array([oracle().compton_energy_from_q(a, b, c) for a, b, c in zip(E, Q, th)])
    ok = (ref_e[:, 1] == 0) & (bad64 == 0)
    nz = ok & (ref_e[:, 0] > 0)
    emi = E - Ii
    h2 = np.sin(th / 2.0) ** 2
    den = np.sqrt(Ii ** 2 + 4.0 * emi * E * h2)
    scale = 137.0 * (2.0 * emi * E * h2 / 510.998928 + Ii) / den  # |numerator| + |binding term|, over den
    live = E > Ii
    small = live & (th < 0.01)
    rel = np.abs(e32[nz] - ref_e[nz, 0]) / ref_e[nz, 0]
    err_q = np.abs(q32 - ref_q)[live] / scale[live]
    err_q_small = np.abs(q32 - ref_q)[small] / scale[small]
    # FP64: the reference's own arithmetic on both sides; fused multiply-adds
    # on the GPU move the results where the reference's forms cancel (the
    # qimax denominator, the discriminant of the quadratic at small angles):
    # measured 9e-11 and 1.5e-9
    err_q64 = (np.abs(q64 - ref_q)[live] / scale[live]).max()
    err_e64 = (np.abs(e64[ok] - ref_e[ok, 0]) / np.maximum(ref_e[ok, 0], 1e-300)).max()
    report = dict(ok=ok.mean(), e32_max=rel.max(), e32_median=np.median(rel), q32_max=err_q.max(),
                  q32_small_max=err_q_small.max(), q64_max=err_q64, e64_max=err_e64)
    print(report)
    assert ok.mean() > 0.99, report
    assert err_q64 < 1e-8 and err_e64 < 1e-8, report
    assert rel.max() < 2e-6 and np.median(rel) < 3e-7, report
    # both signs of Q and both roots are exercised
    assert (nz & (Q > 0)).sum() > 10000 and (nz & (Q < 0)).sum() > 10000
    assert err_q.max() < 2e-6, report
    assert small.sum() > 1000 and err_q_small.max() < 2e-6, report


def analog_cascade_spec(n=100000):
    spec = configs.config1(n_photons_line=n)
    spec.layers = [Layer([82, 26, 8], [0.3, 0.4, 0.3], 6.0, 0.02)]
    spec.reference_layer = 1
    spec.n_interactions_trajectory = 3
    spec.p_detector_window = (0.0, 1.0, 100.0)
    spec.discrete[0].energy = 90.0  # above the Pb K edge
    return spec


@pytest.mark.parametrize("auger,radiative", [(1, 0), (0, 1), (1, 1)])
def test_analog_cascades_fp64_match_oracle(auger, radiative):
    """Variance reduction off with the Auger and/or radiative cascades
    (src/xmi_main.F90:2413-4783): offspring photons in their own slots and
    streams, FP64 GPU against the oracle on the same tables and streams."""
    spec = analog_cascade_spec()
    opts = dict(configs.C1_OPTIONS, use_variance_reduction=0, use_cascade_auger=auger,
                use_cascade_radiative=radiative)
    sim, gpu, ref = run_pair(spec, opts)
    assert gpu["var_red"] is None
    assert_transport_equal(gpu, ref)
    assert gpu["brute"][82 - 1, 29:113, 0].sum() > 0  # Pb L lines
    sim.close()


def test_analog_cascades_fp32_and_batched():
    """FP32 analog transport with both cascades tracks FP64 (1e-2 on the
    brute-force totals: rounding flips a few analog decisions), and a batch of
    an analog cascade configuration with a VR one gives each its single run."""
    spec = analog_cascade_spec(200000)
    opts = dict(configs.C1_OPTIONS, use_variance_reduction=0)
    s64 = Simulation(spec, options=opts, gpu=gpu_options(precision=0, seed=SEED))
    s32 = Simulation(spec, options=opts, gpu=gpu_options(precision=1, seed=SEED))
    r64, r32 = s64.msim(), s32.msim()
    assert r32["brute"].sum() == pytest.approx(r64["brute"].sum(), rel=1e-2)
    pl = slice(29, 113)
    assert r32["brute"][82 - 1, pl].sum() == pytest.approx(r64["brute"][82 - 1, pl].sum(), rel=2e-2)
    np.testing.assert_allclose(r32["channels"].sum(axis=1), r64["channels"].sum(axis=1), rtol=1e-2)
    s64.close()
    s32.close()
    sims = [Simulation(analog_cascade_spec(20000), options=opts, gpu=gpu_options(seed=SEED)),
            Simulation(mixed_source_spec(), options=configs.C1_OPTIONS, gpu=gpu_options(seed=SEED))]
    sims[1].solid_angle()
    batched = Simulation.msim_batch(sims)
    for s, b in zip(sims, batched):
        single = s.msim()
        for key in ("var_red", "brute", "channels"):
            if single[key] is None:
                continue
            np.testing.assert_allclose(b[key], single[key], rtol=1e-9, atol=1e-12 * abs(single[key]).max())
        s.free_raw(b)
        s.free_raw(single)
        s.close()
