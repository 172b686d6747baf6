#!/usr/bin/env python3
"""Benchmark: photon histories/s of the XRF transport on GB300.

Default workload (``--workload batched``): the batched quantification sweep
-- 512 independent sample configurations in the 45/45 geometry of the small
plain configuration (1-8 layers of 2-20 elements, weight fractions +-20%
around the Si/O/Fe/Cu/Zn sample, 1-5 discrete lines or 50-400 intervals of the
Rh-tube spectrum, photon budgets log-uniform in [1e6, 1e8], 4 interactions,
variance reduction on), FP32 transport with FP64 tallies, solid angles from
one surrogate network trained for the detector and shared by all 512, all
configurations in one graph-captured xmi_main_msim_batch call.

One step = one xmi_main_msim_batch call over all 512 configurations with
1/16 of each one's photon budget (``--budget-scale``): the full budgets are
16 steps.
  value  -- histories / device time of the call (CUDA events on its stream:
            transport, event sort, surrogate solid angles, estimator),
  e2e    -- histories / wall time of the public call from the host (source
            items and run descriptors uploaded, tallies copied back and
            reshaped into the reference's output layouts).
  plain  -- the same 512 configurations one by one with the plain GPU method
            (FP32, xmi_solid_angle_calculation grid + xmi_main_msim each):
            the one-by-one transport is timed over all 512, the grid on a
            sample of them; both full jobs (all 16 steps, the network's
            training, every grid) are compared.
  line_error -- the surrogate + batched FP32 output of 32 configurations
            (the 8 with the thinnest layer, the 8 with the heaviest element,
            the rest spread over the budgets) against the all-FP64 plain run
            of the same photons: every line's relative error, every line's
            and every channel's z-score on the combined Monte Carlo standard
            error (estimated from 8 disjoint photon ranges of the FP64 run).

``--workload plain``: the production-size plain configuration -- 5 random
layers (seed 2) of 3-12 elements, Rh tube at 40 kV behind 125 um Be in 400
intervals plus the Rh K/L lines, 6 interactions, one xmi_main_msim per step.

``--workload precision``: the precision form of the small plain
configuration (10 nm Cr and 50 nm Au over a 2 mm substrate, 1e8 photons per
step), FP32 transport timed, with the error of every line and channel against
the all-FP64 run of the same photons (relative error and z-score on the
Monte Carlo standard error from disjoint photon ranges).

``--workload surrogate``: the learned solid-angle surrogate on its own
geometry -- the small plain configuration behind a conical collimator
(height 1 cm, opening radius 0.1 cm), 1e8 photons per step, FP32 transport.
The grid path (a 1000 x 1000 FP64 grid, then the transport reading it) and
the surrogate path (the network trained on 2e6 integrator samples uniform
over the sample volume, checked per cell at the 1e-3 tolerance, flagged
cells served by the tabulated integrator, then the transport serving it)
are both timed; the line is the surrogate path's, with the network's check,
a held-out validation at the estimator's own query points and the per-line
error against the grid path beside it.

Multi-GPU (torchrun): every rank runs its own configurations (weak scaling,
no data-path collective); with --partition the ranks split one batched sweep,
whole configurations balanced by budget (strong scaling; the configuration
outputs are each one rank's, the same as a single process's).  The job's
value is the histories of all ranks over the slowest rank's time.

``--impl reference`` times the reference algorithm's CPU path: the FP64 C
restatement under oracle/ (the reference's Fortran build needs gfortran and
xraylib, absent here) with all host threads, each step a bounded sample of
the same workload: every configuration of the sweep, each source item
running the same share of its photons (1e6 photons in all by default), one
call per configuration as the reference runs them.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "photon histories/s on 1 GB300: surrogate+batched vs plain, at <=0.5% line error"
PLAIN_METRIC = "photon histories/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="batched", choices=["batched", "plain", "surrogate", "precision"])
    p.add_argument("--plain-mode", default="default", choices=["default", "advanced-compton", "analog"],
                   help="transport options of the plain workload")
    p.add_argument("--configs", type=int, default=512, help="configurations of the batched workload")
    p.add_argument("--budget-scale", type=float, default=1.0 / 16, help="share of each budget per step")
    p.add_argument("--n-train", type=int, default=1 << 21, help="integrator samples the surrogate trains on")
    p.add_argument("--epochs", type=int, default=8)
    p.add_argument("--tolerance", type=float, default=1e-3, help="surrogate held-out error limit")
    p.add_argument("--hits-check", type=int, default=1 << 19, help="FP64 integrator samples per checking point")
    p.add_argument("--plain-grids", type=int, default=4, help="grids timed for the plain comparison")
    p.add_argument("--tune-share", type=float, default=1.0 / 32, help="share of a step the autotuner's trials run")
    p.add_argument("--queue-events", type=int, default=0,
                   help="skip the autotuner: default launch shape and this estimator queue size (small profiling runs)")
    p.add_argument("--line-configs", type=int, default=32, help="configurations of the FP64 error statement")
    p.add_argument("--replicas", type=int, default=8,
                   help="disjoint photon ranges of the FP64 reference runs (their spread is the MC error)")
    p.add_argument("--overlap-chunks", type=int, default=0,
                   help="1: the next chunk's transport beside the current chunk's sort, solid angles and estimator")
    p.add_argument("--estimator-blocks-per-sm", type=int, default=0, help="estimator blocks per SM (0: as many as fit)")
    p.add_argument("--partition", action="store_true",
                   help="batched workload on N ranks: one sweep, whole configurations split by budget "
                        "(strong scaling) instead of a sweep per rank (weak scaling)")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--photons", type=float, default=1e7, help="photons per step of the plain workload")
    p.add_argument("--photons-precision", type=float, default=1e8, help="photons per step of the precision workload")
    p.add_argument("--photons-surrogate", type=float, default=1e8,
                   help="photons per step of the surrogate workload")
    p.add_argument("--hits-train", type=int, default=1 << 14,
                   help="integrator samples per training point of the surrogate workload")
    p.add_argument("--epochs-surrogate", type=int, default=32, help="training epochs of the surrogate workload")
    p.add_argument("--n-train-surrogate", type=int, default=2_000_000,
                   help="training points of the surrogate workload (uniform over the sample volume)")
    p.add_argument("--surrogate-points", default="volume", choices=["volume", "pilot"],
                   help="surrogate workload: train on points uniform over the sample volume (the workload's "
                        "definition) or on the estimator's query points of a pilot run")
    p.add_argument("--precision", default="fp32", choices=["fp64", "fp32"])
    p.add_argument("--cpu-sample", type=int, default=1000000,
                   help="photons of the CPU-baseline sample (spread over all configurations by budget)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def histories(spec) -> int:
    """Photon histories one xmi_main_msim of spec simulates (src/xmi_main.F90:240-858)."""
    return int(spec.n_photons_interval) * max(0, len(spec.continuous) - 1) + \
        int(spec.n_photons_line) * len(spec.discrete)


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
PLAIN_MODES = {
    "default": "VR on, Doppler Compton",
    "advanced-compton": "VR on, per-shell impulse-approximation Compton (use_advanced_compton = 1)",
    "analog": "VR off, analog Auger and radiative cascades",
}


def plain_workload(photons: float, mode: str = "default"):
    from xmimsim_gb300 import configs
    spec = configs.config2(total_photons=int(photons))
    options = dict(configs.C2_OPTIONS, use_sum_peaks=0)
    if mode == "advanced-compton":
        options["use_advanced_compton"] = 1
    elif mode == "analog":
        options.update(use_variance_reduction=0, use_cascade_auger=1, use_cascade_radiative=1)
    return spec, options


def batched_specs(n: int, scale: float, rank: int = 0):
    from xmimsim_gb300 import configs
    return configs.config5(n, seed=5 + 1000 * rank, budget_scale=scale), dict(configs.C5_OPTIONS)


def total_thickness(spec) -> float:
    return sum(l.thickness for l in spec.layers)


# --------------------------------------------------------------------------
# CPU baseline (the oracle: FP64 restatement of the reference's algorithm)
# --------------------------------------------------------------------------
class CpuSample:
    """The FP64 CPU restatement (all threads) on a bounded, budget-weighted
    sample of a workload: every configuration runs the same share of each of
    its source items' photons (about n_sample photons in all), so the sample
    has the workload's own mix of configurations.  The set-up (tables, and a
    coarse 64 x 64 solid-angle grid of 500 samples per point built by the
    CPU integrator so that no GPU is needed) is done once and not timed."""

    def __init__(self, specs, options, n_sample: int):
        from oracle import oracle_api
        from xmimsim_gb300 import Simulation, gpu_options
        import numpy as np
        self.O = oracle_api
        total = sum(histories(sp) for sp in specs)
        self.share = min(1.0, n_sample / max(1, total))
        self.sims, self.items = [], []
        for spec in specs:
            sim = Simulation(spec, options=options, gpu=gpu_options(seed=0x5EED0001))
            r, t = sim.grid_axes(64, 64)
            sim.set_solid_angle(r, t, np.zeros((64, 64)))
            sim.prepare()
            g = oracle_api.solid_angle_points(sim.bundle_ptr(), r, t, 0, 64 * 64, 500).reshape(64, 64)
            sim.set_solid_angle(r, t, g)
            sim.prepare()
            per_item = max(1, int(round(max(int(spec.n_photons_line), int(spec.n_photons_interval)) * self.share)))
            n = min(per_item, int(spec.n_photons_line)) * len(spec.discrete) + \
                min(per_item, int(spec.n_photons_interval)) * max(0, len(spec.continuous) - 1)
            self.sims.append(sim)
            self.items.append((spec, per_item, n))
        self.n_hist = sum(n for _, _, n in self.items)

    def run(self, threads: int):
        """One timed pass: (histories/s, histories, seconds, words/history of
        transport, words/history of the estimator loops)."""
        dt, words_tr, words_est = 0.0, 0, 0
        for sim, (spec, per_item, _) in zip(self.sims, self.items):
            self.O.words_counted_split()
            t0 = time.perf_counter()
            self.O.msim(sim.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels, threads=threads,
                        max_photons_per_item=per_item)
            dt += time.perf_counter() - t0
            w, we = self.O.words_counted_split()
            words_tr += w - we
            words_est += we
        return self.n_hist / dt, self.n_hist, dt, words_tr / self.n_hist, words_est / self.n_hist

    def close(self):
        for sim in self.sims:
            sim.close()


def run_cpu_sample(specs, options, n_sample: int, threads: int):
    cs = CpuSample(specs, options, n_sample)
    try:
        return cs.run(threads)
    finally:
        cs.close()


def cpu_sample_specs(args, rank=0):
    if args.workload == "plain":
        spec, options = plain_workload(args.photons, args.plain_mode)
        return [spec], options, "the %.0e-photon plain workload" % args.photons
    if args.workload == "surrogate":
        from xmimsim_gb300 import configs
        return [configs.config4(int(args.photons_surrogate))], dict(configs.C1_OPTIONS), \
            "the collimated surrogate workload"
    if args.workload == "precision":
        from xmimsim_gb300 import configs
        return [configs.config3(int(args.photons_precision))], dict(configs.C1_OPTIONS), \
            "the thin-layer precision workload"
    specs, options = batched_specs(args.configs, args.budget_scale, rank)
    return specs, options, "all %d batched configurations, each item's photons in the step's proportions" % len(specs)


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    specs, options, what = cpu_sample_specs(args)
    threads = os.cpu_count() or 1
    vals = []
    cs = CpuSample(specs, options, args.cpu_sample)
    for i in range(args.warmup + args.steps):
        v, n, dt, _, _ = cs.run(threads)
        if i >= args.warmup:
            vals.append((v, n, dt))
    cs.close()
    value = statistics.median(v for v, _, _ in vals)
    sample = "%d photons per step over %s" % (vals[0][1], what)
    batched = args.workload == "batched"
    line = {"metric": METRIC if batched else PLAIN_METRIC, "value": value, "unit": "histories/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(d for _, _, d in vals) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random samples, Rh tube spectrum / discrete lines)",
            "config": workload_config(args, None),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_config(args, extra):
    if args.workload == "precision":
        cfg = {"workload": "precision form of config 1: 10 nm Cr and 50 nm Au over a 2 mm substrate, FP32 transport "
                           "and tables, FP64 positions and tallies, error statement against all-FP64",
               "photons_per_step": int(args.photons_precision)}
    elif args.workload == "surrogate":
        cfg = {"workload": "collimated config-1 geometry (conical collimator 1 cm high, 0.1 cm opening radius, "
                           "45/45 degrees, 10 cm), FP32 transport, solid angles from the surrogate network",
               "photons_per_step": int(args.photons_surrogate)}
    elif args.workload == "plain":
        cfg = {"workload": "plain 5-layer Rh 40 kV, 400 intervals + Rh K/L lines, 6 interactions, "
                           + PLAIN_MODES[args.plain_mode],
               "photons_per_step": int(args.photons)}
    else:
        cfg = {"workload": "%d-configuration quantification sweep: 1-8 layers of 2-20 elements, 1-5 lines or "
                           "50-400 Rh-tube intervals, budgets log-uniform 1e6-1e8, 4 interactions, VR on, "
                           "FP32 + shared surrogate, one graph-captured batched call" % args.configs,
               "configs": args.configs, "budget_share_per_step": args.budget_scale,
               "steps_per_full_job": round(1.0 / args.budget_scale)}
    if extra:
        cfg.update(extra)
    return cfg


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def load_cudart():
    import ctypes as C
    try:
        return C.CDLL("libcudart.so")
    except OSError:
        import glob
        c = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        return C.CDLL(c[0]) if c else None


def timed_steps(args, step, local):
    """W untimed steps, then K timed ones between device synchronisations;
    returns (per-step timing dicts, wall seconds, clocks summary)."""
    cudart = load_cudart()
    for _ in range(args.warmup):
        step()
    if cudart is not None:
        cudart.cudaDeviceSynchronize()
    tms = []
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            tms.append(step())
        if cudart is not None:
            cudart.cudaDeviceSynchronize()
        wall = time.perf_counter() - t0
    return tms, wall, clocks.summary()


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per history of
# one estimator_kernel launch, from ncu captures of the FP32 kernel: the
# batched sweep's small case (16 configurations, a 2^20-photon chunk:
# 304.9 + 17.1 MB) and the plain production workload (1e6 photons: 393.9 +
# 15.2 MB).  Traffic grows in proportion to the histories of a launch.
ESTIMATOR_DRAM_BYTES_PER_HISTORY = {"batched": 322.0e6 / 1048576, "plain": 409.1e6 / 1.0e6}


def roofline_block(ph_ms: dict, n_hist_per_step: int, words_tr: float, words_est: float, word: int,
                   traffic_per_history: float | None = None, hist_per_launch: float | None = None):
    """Dominant kernel: algorithmic table bytes it reads per history (counted
    by the instrumented oracle on the CPU sample) over its device time;
    traffic: measured DRAM bytes of one launch (per-history figure scaled to
    the histories of one launch of this run)."""
    kern = "estimator_kernel" if ph_ms["estimator"] >= ph_ms["transport"] else "wf_step + wf_interact"
    kms = ph_ms["estimator"] if kern == "estimator_kernel" else ph_ms["transport"]
    bph = (words_est if kern == "estimator_kernel" else words_tr) * word
    pk = peaks()
    peak = pk.get("hbm_gbs", 6800.0)
    achieved = bph * n_hist_per_step / (kms / 1e3) / 1e9 if kms > 0 else 0.0
    traffic = None
    if kern == "estimator_kernel" and traffic_per_history and hist_per_launch:
        traffic = traffic_per_history * hist_per_launch
    return {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_per_history": traffic_per_history,
            "algorithmic_bytes_per_history": bph,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one estimator launch "
                              "(small case of this workload), scaled to this run's histories per launch",
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if pk else "fallback 6.8 TB/s"}


def line_error(sur_out: dict, ref_out: dict, floor: float = 1e-2) -> dict:
    """Relative error of every line (summed over interaction orders) carrying
    at least `floor` of the configuration's strongest line."""
    import numpy as np
    a = sur_out["var_red"].sum(axis=2).ravel()
    b = ref_out["var_red"].sum(axis=2).ravel()
    bad = int((~np.isfinite(a)).sum() + (~np.isfinite(b)).sum())
    if bad:
        return {"nonfinite": bad}
    m = b > floor * b.max()
    rel = np.abs(a[m] - b[m]) / b[m]
    return {"lines": int(m.sum()), "max": float(rel.max()) if m.any() else 0.0,
            "median": float(np.median(rel)) if m.any() else 0.0,
            "within_0.5pct": float((rel <= 5e-3).mean()) if m.any() else 1.0,
            "total": float(abs(a.sum() - b.sum()) / b.sum()) if b.sum() > 0 else 0.0}


def replica_runs(sim, k_rep: int):
    """The run as k_rep disjoint photon ranges (xmi_gpu_set_replica, each with
    the full budget's weights): their sum is the full run and their spread
    its Monte Carlo error.  Returns (lines [k, 100, 385, N], channels
    [k, N + 1, nch])."""
    import numpy as np
    lines, chans = [], []
    for k in range(k_rep):
        sim.set_replica(k, k_rep)
        o = sim.msim()
        lines.append(o["var_red"].copy())
        chans.append(o["channels"].copy())
        sim.free_raw(o)
    sim.set_replica(0, 1)
    return np.array(lines), np.array(chans)


def error_statement(out32: dict, reps64: tuple, strong: float = 1e-3, floor: float = 1e-9) -> dict:
    """Error of an FP32 run against the all-FP64 run of the same photons, for
    every line and every channel.  reps64: the FP64 run as k replicas
    (replica_runs); its sum is the reference and k times the variance of the
    replicas its Monte Carlo variance.  The combined standard error of two
    independent runs of this size is sqrt(2) sigma_64; z = (FP32 - FP64) /
    that.  Lines are summed over orders; channels are every order's spectrum
    (cumulative rows 1..N).

    The relative and z statistics cover the resolved entries: lines at least
    `floor` of the strongest line, channels at least `floor` of their order's
    largest channel.  Below that an entry is no measurable signal (FP32
    underflows the attenuation of lines 1e-40 below the strongest, and a
    single event that takes another Compton energy in FP32 than in FP64 can
    dominate a channel that holds 1e-12 of the spectrum); those are counted,
    and every entry's absolute difference is given relative to the strongest
    line / channel.  The entries furthest from the FP64 run in sigma are
    listed."""
    import numpy as np
    l64k, c64k = reps64
    k = l64k.shape[0]
    a = out32["var_red"].sum(axis=2)
    lk = l64k.sum(axis=3)
    b, sb = lk.sum(axis=0), np.sqrt(k * lk.var(axis=0, ddof=1))
    if not (np.isfinite(a).all() and np.isfinite(b).all()):
        return {"nonfinite": int((~np.isfinite(a)).sum() + (~np.isfinite(b)).sum())}
    bmax = b.max() if b.max() > 0 else 1.0
    m = b >= floor * bmax
    rel = np.abs(a[m] - b[m]) / b[m]
    st = (b >= strong * bmax)[m]
    zm = m & (sb > 0)
    z = (a[zm] - b[zm]) / (np.sqrt(2.0) * sb[zm])
    ca = out32["channels"][1:]
    cb, scb = c64k.sum(axis=0)[1:], np.sqrt(k * c64k.var(axis=0, ddof=1))[1:]
    cmax = np.maximum(np.abs(cb).max(axis=1, keepdims=True), 1e-300)
    cm = (scb > 0) & (np.abs(cb) >= floor * cmax)
    zc = (ca[cm] - cb[cm]) / (np.sqrt(2.0) * scb[cm])
    zl = np.zeros_like(b)
    zl[zm] = z
    worst_l = []
    for flat in np.argsort(-np.abs(zl).ravel())[:3]:
        zi, li = np.unravel_index(flat, b.shape)
        if zl[zi, li] != 0:
            worst_l.append({"Z": int(zi + 1), "line": int(li + 1), "fp64": float(b[zi, li]),
                            "rel": float((a[zi, li] - b[zi, li]) / b[zi, li]), "z": float(zl[zi, li]),
                            "sigma_rel": float(sb[zi, li] / b[zi, li]), "share": float(b[zi, li] / bmax)})
    zcf = np.zeros_like(cb)
    zcf[cm] = zc
    worst_c = []
    for flat in np.argsort(-np.abs(zcf).ravel())[:3]:
        oi, ci = np.unravel_index(flat, cb.shape)
        if zcf[oi, ci] != 0:
            worst_c.append({"order": int(oi + 1), "channel": int(ci), "fp64": float(cb[oi, ci]),
                            "rel": float((ca[oi, ci] - cb[oi, ci]) / cb[oi, ci]), "z": float(zcf[oi, ci]),
                            "sigma_rel": float(scb[oi, ci] / abs(cb[oi, ci]))})
    return {"lines": int(m.sum()), "lines_unresolved": int(((b > 0) & ~m).sum()),
            "lines_max_rel": float(rel.max()) if m.any() else 0.0,
            "lines_median_rel": float(np.median(rel)) if m.any() else 0.0,
            "lines_within_0.5pct": float((rel <= 5e-3).mean()) if m.any() else 1.0,
            "strong_lines": int(st.sum()), "strong_max_rel": float(rel[st].max()) if st.any() else 0.0,
            "strong_within_0.5pct": float((rel[st] <= 5e-3).mean()) if st.any() else 1.0,
            "lines_with_sigma": int(zm.sum()),
            "lines_within_3sigma": float((np.abs(z) <= 3).mean()) if len(z) else 1.0,
            "lines_max_abs_z": float(np.abs(z).max()) if len(z) else 0.0,
            "lines_max_abs_diff_over_strongest": float(np.abs(a - b).max() / bmax),
            "channels_with_sigma": int(cm.sum()),
            "channels_unresolved": int(((scb > 0) & ~cm).sum()),
            "channels_within_3sigma": float((np.abs(zc) <= 3).mean()) if len(zc) else 1.0,
            "channels_max_abs_z": float(np.abs(zc).max()) if len(zc) else 0.0,
            "channels_max_abs_diff_over_max": float((np.abs(ca - cb) / cmax).max()),
            "total_rel": float(abs(a.sum() - b.sum()) / b.sum()) if b.sum() > 0 else 0.0,
            "floor": floor, "replicas": int(k), "worst_lines": worst_l, "worst_channels": worst_c}


def merge_statements(parts: list[dict]) -> dict:
    """Worst case (max) and pooled fractions of several error statements."""
    parts = [p for p in parts if "lines" in p]
    if not parts:
        return {}
    out = {"configs": len(parts)}
    for key in ("lines_max_rel", "strong_max_rel", "lines_max_abs_z", "channels_max_abs_z", "total_rel",
                "lines_max_abs_diff_over_strongest", "channels_max_abs_diff_over_max"):
        out[key] = max(p[key] for p in parts)
    for key in ("lines_unresolved", "channels_unresolved"):
        out[key] = sum(p[key] for p in parts)
    for frac, count in (("lines_within_0.5pct", "lines"), ("strong_within_0.5pct", "strong_lines"),
                        ("lines_within_3sigma", "lines_with_sigma"), ("channels_within_3sigma", "channels_with_sigma")):
        n = sum(p[count] for p in parts)
        out[frac] = sum(p[frac] * p[count] for p in parts) / n if n else 1.0
        out[count] = n
    return out


def batched_arm(args, ws, rank, local):
    import numpy as np
    from xmimsim_gb300 import Simulation, gpu_options, last_timing
    # weak scaling: a sweep of its own per rank; --partition: one sweep, each
    # rank runs its share of whole configurations (balanced by budget) with
    # the same photon streams as a single process would
    part = args.partition and ws > 1
    sweep_rank = 0 if args.partition else rank
    specs, options = batched_specs(args.configs, args.budget_scale, sweep_rank)
    full_specs, _ = batched_specs(args.configs, 1.0, sweep_rank)
    if part:
        from xmimsim_gb300.replicas import rank_share
        mine = rank_share(specs, rank, ws)
        specs, full_specs = [specs[i] for i in mine], [full_specs[i] for i in mine]
    seed = 0x5EED0005 + sweep_rank
    g_sur = gpu_options(precision=1, seed=seed, use_surrogate=1, surrogate_tolerance=args.tolerance,
                        overlap_chunks=args.overlap_chunks, estimator_blocks_per_sm=args.estimator_blocks_per_sm)
    t0 = time.perf_counter()
    sims = [Simulation(s, options=options, gpu=g_sur) for s in specs]
    host_tables_s = time.perf_counter() - t0
    n_hist = sum(histories(s) for s in specs)
    full_hist = sum(histories(s) for s in full_specs)

    # one network for the detector, trained where the estimator queries solid
    # angles: points from pilot runs of 8 configurations (the deepest sample
    # and 7 spread over the sweep)
    import numpy as np
    deep = max(range(len(specs)), key=lambda i: total_thickness(specs[i]))
    pick = sorted(set([deep] + [int(i) for i in np.linspace(0, len(specs) - 1, 7)]))
    t0 = time.perf_counter()
    per = (args.n_train + (1 << 14)) // len(pick) + 1
    rs, ts = [], []
    for i in pick:
        share = min(1.0, 2.0 * per / max(1, histories(specs[i])))
        r, t = sims[i].sample_event_points(share, per)
        rs.append(r)
        ts.append(t)
    pilot_s = time.perf_counter() - t0
    rep = sims[deep].build_surrogate_points(np.concatenate(rs), np.concatenate(ts), hits_train=1024,
                                            epochs=args.epochs, hits_check=args.hits_check)
    rep["pilot_s"] = pilot_s
    rep["pilot_configs"] = len(pick)
    train_s = time.perf_counter() - t0
    for i, s in enumerate(sims):
        if i != deep:
            s.share_surrogate(sims[deep])
    # launch shape and queue size of the batched call
    t0 = time.perf_counter()
    if args.queue_events:
        # fixed shape (small profiling runs): default launch shape, given queue size
        for s in sims:
            s.gpu.queue_events = args.queue_events
            s.set_gpu(s.gpu)
        tune = {"threads_per_block": 128, "blocks_per_sm": 8, "queue_events": args.queue_events,
                "best_trial_ms": None, "share": 0.0}
    else:
        tune = Simulation.autotune_batch(sims, share=args.tune_share)
    tune["wall_s"] = time.perf_counter() - t0

    last = {}

    def step():
        outs = Simulation.msim_batch(sims, copy=False)
        tm = last_timing()
        if "outs" in last:
            for s, o in zip(sims, last["outs"]):
                s.free_raw(o)
        last["outs"] = outs
        return tm

    tms, wall, clocks = timed_steps(args, step, local)
    ksum = sum(t["kernel_ms"] for t in tms)
    value = n_hist * args.steps / (ksum / 1e3)
    e2e = n_hist * args.steps / wall
    phases = {k: statistics.mean(t[k + "_ms"] for t in tms) for k in ("transport", "sort", "surrogate", "estimator")}
    extra = {"photons_per_step": n_hist, "photons_full_job": full_hist,
             "ranks": ("one sweep, %d of its configurations on this rank (whole configurations balanced by "
                       "budget)" % len(specs)) if part else "a sweep per rank",
             "elements_per_config_mean": statistics.mean(sum(len(l.Z) for l in s.layers) for s in specs),
             "l2": "inputs larger than L2 (tables of 512 configurations, several GB)",
             "host_tables_s": host_tables_s, "autotuned": tune,
             "surrogate": dict(rep, n_train=args.n_train, epochs=args.epochs, tolerance=args.tolerance,
                              hits_check=args.hits_check, wall_s=train_s)}
    line = {"metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ksum / args.steps, "higher_is_better": True,
            "scaling": "strong" if part else "weak",
            "vs_baseline": None, "dtype": "f32 transport, f64 tallies",
            "data": "synthetic (seeded random samples, Rh tube spectrum / discrete lines)",
            "config": workload_config(args, extra),
            "gpu_launches": sum(t["launches"] for t in tms),
            "phases_ms_per_step": phases,
            "events_per_step": statistics.mean(t["events"] for t in tms),
            "surrogate_fallbacks_per_step": statistics.mean(t["surrogate_fallbacks"] for t in tms),
            "e2e": {"value": e2e, "unit": "histories/s",
                    "h2d_bytes_per_step": int(statistics.mean(t["h2d_bytes"] for t in tms)),
                    "d2h_bytes_per_step": int(statistics.mean(t["d2h_bytes"] for t in tms))},
            "clocks": clocks}
    steps_full = 1.0 / args.budget_scale
    sb_full_s = train_s + steps_full * wall / args.steps

    if not args.no_plain:
        sb = {"full_job_s": sb_full_s, "full_job_histories_per_s": full_hist / sb_full_s,
              "includes": "network training + autotuning + %d batched steps (wall)" % round(steps_full)}
        line["surrogate_batched_full_job"] = sb
        line["plain"] = {}
        for prec, name in ((0, "fp64"), (1, "fp32")):
            line["plain"][name] = one_by_one(args, sims, specs, options, deep, seed, prec, tune, n_hist,
                                             full_hist, steps_full)
        # the plain GPU method: all-FP64 transport and grid, one configuration per call
        line["speedup_full_job_vs_plain"] = line["plain"]["fp64"]["full_job_s"] / sb_full_s
        line["speedup_full_job_vs_fp32_one_by_one"] = line["plain"]["fp32"]["full_job_s"] / sb_full_s
        for s in sims:
            s.set_gpu(g_sur)

    if args.line_configs > 0 and "outs" in last:
        # the all-FP64 plain run (FP64 transport on an FP64 grid, same photon
        # streams) of line_configs configurations: the 8 with the thinnest
        # layer, the 8 with the heaviest element and the rest spread over the
        # budgets; each as args.replicas disjoint photon ranges for its
        # Monte Carlo error
        t0 = time.perf_counter()
        by_thin = sorted(range(len(specs)), key=lambda i: min(l.thickness for l in specs[i].layers))
        by_heavy = sorted(range(len(specs)), key=lambda i: -max(max(l.Z) for l in specs[i].layers))
        by_budget = sorted(range(len(specs)), key=lambda i: histories(specs[i]))
        pick = []
        for i in by_thin[:8] + by_heavy[:8]:
            if i not in pick:
                pick.append(i)
        n_spread = max(0, args.line_configs - len(pick))
        for k in range(n_spread):
            i = by_budget[len(by_budget) * (2 * k + 1) // (2 * n_spread)]
            if i not in pick:
                pick.append(i)
        g64 = gpu_options(precision=0, seed=seed)
        gd = Simulation(specs[deep], options=options, gpu=g64)
        ax64 = gd.solid_angle_grid()
        gd.close()
        parts = []
        for i in pick:
            ref = Simulation(specs[i], options=options, gpu=g64)
            ref.set_solid_angle(ax64["r"], ax64["theta"], ax64["grid"])
            e = error_statement(last["outs"][i], replica_runs(ref, args.replicas))
            e.update(config=int(i), photons=histories(specs[i]),
                     thinnest_cm=min(l.thickness for l in specs[i].layers),
                     heaviest_Z=max(max(l.Z) for l in specs[i].layers))
            parts.append(e)
            ref.close()
        line["line_error"] = {"reference": "all-FP64 plain GPU run (FP64 transport, FP64 grid of the deepest "
                                           "sample), same photon streams",
                              "summary": merge_statements(parts), "configs": parts,
                              "wall_s": time.perf_counter() - t0}
    if "outs" in last:
        for s, o in zip(sims, last["outs"]):
            s.free_raw(o)
    return line, sims, specs, options


def one_by_one(args, sims, specs, options, deep, seed, prec, tune, n_hist, full_hist, steps_full):
    """The configurations one by one, each with its own solid-angle grid and
    one xmi_main_msim call, in the given precision.  Grids are timed on
    `--plain-grids` configurations; the transport on every configuration
    (FP32) or every k-th one (FP64, scaled by photons), after an untimed pass
    over 1/1000 of the photons that puts tables and grids on the device.  The
    transport runs on the deepest sample's grid (axes spanning every other's)."""
    import numpy as np
    from xmimsim_gb300 import Simulation, gpu_options
    g = gpu_options(precision=prec, seed=seed, threads_per_block=tune["threads_per_block"],
                    blocks_per_sm=tune["blocks_per_sm"])
    g.queue_events = tune["queue_events"]
    grid_s = []
    for i in np.linspace(0, len(sims) - 1, args.plain_grids).astype(int):
        ps = Simulation(specs[i], options=options, gpu=g)
        t0 = time.perf_counter()
        ps.solid_angle()
        grid_s.append(time.perf_counter() - t0)
        ps.close()
    gd = Simulation(specs[deep], options=options, gpu=g)
    ax = gd.solid_angle_grid()
    gd.close()
    k = 1 if prec == 1 else max(1, len(sims) // 128)
    sub = sims[::k]
    for s in sub:
        s.set_gpu(g)
        s.set_solid_angle(ax["r"], ax["theta"], ax["grid"])
        s.set_replica(0, 1000)
        s.free_raw(s.msim())
        s.set_replica(0, 1)
    load_cudart().cudaDeviceSynchronize()
    t0 = time.perf_counter()
    dev_ms = 0.0
    for s in sub:
        o = s.msim()
        dev_ms += s.timing()["kernel_ms"]
        s.free_raw(o)
    wall = time.perf_counter() - t0
    n_sub = sum(histories(specs[i]) for i in range(0, len(sims), k))
    step_s = wall * n_hist / n_sub
    full_s = len(sims) * statistics.mean(grid_s) + steps_full * step_s
    return {"method": "one xmi_solid_angle_calculation grid + one xmi_main_msim per configuration, %s"
                      % ("all FP64" if prec == 0 else "FP32 transport, FP64 tallies"),
            "value": n_sub / wall, "unit": "histories/s", "device_value": n_sub / (dev_ms / 1e3),
            "note": "value: one-by-one transport (wall, grids excluded) over %d of %d configurations"
                    % (len(sub), len(sims)),
            "grid_s_per_config": statistics.mean(grid_s), "grids_timed": len(grid_s),
            "full_job_s": full_s, "full_job_histories_per_s": full_hist / full_s}


def plain_arm(args, ws, rank, local):
    from xmimsim_gb300 import Simulation, gpu_options
    spec, options = plain_workload(args.photons, args.plain_mode)
    precision = 0 if args.precision == "fp64" else 1
    t0 = time.perf_counter()
    sim = Simulation(spec, options=options, gpu=gpu_options(precision=precision, seed=0x5EED0001 + rank))
    sim.solid_angle()
    grid_s = time.perf_counter() - t0
    n_hist = histories(spec)

    def step():
        out = sim.msim()
        tm = sim.timing()
        sim.free_raw(out)
        return tm

    tms, wall, clocks = timed_steps(args, step, local)
    ksum = sum(t["kernel_ms"] for t in tms)
    line = {"metric": PLAIN_METRIC, "value": n_hist * args.steps / (ksum / 1e3), "unit": "histories/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ksum / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if precision == 0 else "f32 transport, f64 tallies",
            "data": "synthetic (seeded random 5-layer sample, Rh tube spectrum)",
            "config": workload_config(args, {"elements": sum(len(l.Z) for l in spec.layers),
                                             "l2": "inputs larger than L2 (angular tables exceed 129 MB)",
                                             "solid_angle_grid_s": grid_s}),
            "gpu_launches": sum(t["launches"] for t in tms),
            "phases_ms_per_step": dict({k: statistics.mean(t[k + "_ms"] for t in tms)
                                        for k in ("transport", "sort", "estimator")},
                                       off_grid_solid_angles=statistics.mean(t["surrogate_ms"] for t in tms)),
            "events_per_step": statistics.mean(t["events"] for t in tms),
            "e2e": {"value": n_hist * args.steps / wall, "unit": "histories/s",
                    "h2d_bytes_per_step": int(statistics.mean(t["h2d_bytes"] for t in tms)),
                    "d2h_bytes_per_step": int(statistics.mean(t["d2h_bytes"] for t in tms))},
            "clocks": clocks}
    return line, [sim], [spec], options


def precision_arm(args, ws, rank, local):
    """The precision workload: thin layers (10 nm Cr, 50 nm Au) over a 2 mm
    substrate in the config-1 geometry, FP32 transport timed, and its error
    statement against the all-FP64 run of the same photons (same FP64 grid)."""
    from xmimsim_gb300 import Simulation, configs, gpu_options
    spec = configs.config3(n_photons_line=int(args.photons_precision))
    options = dict(configs.C1_OPTIONS)
    seed = 0x5EED0003 + rank
    n_hist = histories(spec)
    g64 = gpu_options(precision=0, seed=seed)
    ref = Simulation(spec, options=options, gpu=g64)
    ax = ref.solid_angle_grid()
    sim = Simulation(spec, options=options, gpu=gpu_options(precision=1, seed=seed))
    sim.set_solid_angle(ax["r"], ax["theta"], ax["grid"])
    last = {}

    def step():
        out = sim.msim()
        tm = sim.timing()
        if "out" in last:
            sim.free_raw(last["out"])
        last["out"] = out
        return tm

    tms, wall, clocks = timed_steps(args, step, local)
    ksum = sum(t["kernel_ms"] for t in tms)
    t0 = time.perf_counter()
    err = error_statement(last["out"], replica_runs(ref, args.replicas))
    ref_s = time.perf_counter() - t0
    sim.free_raw(last["out"])
    ref.close()
    line = {"metric": PLAIN_METRIC + " (FP32 transport, thin layers)", "value": n_hist * args.steps / (ksum / 1e3),
            "unit": "histories/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ksum / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 transport, f64 tallies", "data": "synthetic (config-1 sample under 10 nm Cr and 50 nm Au)",
            "config": workload_config(args, {"layers_cm": [l.thickness for l in spec.layers]}),
            "gpu_launches": sum(t["launches"] for t in tms),
            "phases_ms_per_step": dict({k: statistics.mean(t[k + "_ms"] for t in tms)
                                        for k in ("transport", "sort", "estimator")},
                                       off_grid_solid_angles=statistics.mean(t["surrogate_ms"] for t in tms)),
            "events_per_step": statistics.mean(t["events"] for t in tms),
            "e2e": {"value": n_hist * args.steps / wall, "unit": "histories/s",
                    "h2d_bytes_per_step": int(statistics.mean(t["h2d_bytes"] for t in tms)),
                    "d2h_bytes_per_step": int(statistics.mean(t["d2h_bytes"] for t in tms))},
            "error_vs_fp64": dict(err, reference="all-FP64 run of the same photons and grid, %d replicas (%.1f s)"
                                  % (args.replicas, ref_s)),
            "clocks": clocks}
    return line, [sim], [spec], options


def surrogate_arm(args, ws, rank, local):
    """The collimated surrogate workload: grid path and surrogate path on the
    same photon streams."""
    import numpy as np
    from xmimsim_gb300 import Simulation, configs, gpu_options
    spec = configs.config4(n_photons_line=int(args.photons_surrogate))
    options = dict(configs.C1_OPTIONS)
    seed = 0x5EED0004 + rank
    n_hist = histories(spec)
    cudart = load_cudart()

    # grid path: the reference-style 1000 x 1000 grid, FP64 integrator
    g64 = gpu_options(precision=0, seed=seed, grid_n=1000)
    gsim = Simulation(spec, options=options, gpu=g64)
    t0 = time.perf_counter()
    ax = gsim.solid_angle_grid()
    grid_s = time.perf_counter() - t0
    grid_run = Simulation(spec, options=options, gpu=gpu_options(precision=1, seed=seed, grid_n=1000))
    grid_run.set_solid_angle(ax["r"], ax["theta"], ax["grid"])

    # surrogate path: 2e6 training samples uniform over the sample volume
    g_sur = gpu_options(precision=1, seed=seed, use_surrogate=1, surrogate_tolerance=args.tolerance, grid_n=1000)
    sur = Simulation(spec, options=options, gpu=g_sur)
    t0 = time.perf_counter()
    if args.surrogate_points == "pilot":
        pil = Simulation(spec, options=options, gpu=gpu_options(precision=1, seed=seed ^ 0x1234, use_surrogate=1))
        pr, pt = pil.sample_event_points(share=min(1.0, 2.0 * args.n_train_surrogate / n_hist),
                                         max_points=args.n_train_surrogate)
        pil.close()
        rep = sur.build_surrogate_points(pr, pt, hits_train=args.hits_train, epochs=args.epochs_surrogate,
                                         hits_check=args.hits_check)
    else:
        rep = sur.build_surrogate(n_train=args.n_train_surrogate, hits_train=args.hits_train,
                                  epochs=args.epochs_surrogate, hits_check=args.hits_check)
    train_s = time.perf_counter() - t0
    # held-out validation at the estimator's own query points (a pilot run
    # with another seed), judged by the integrator with 2^24 samples per point
    pilot = Simulation(spec, options=options, gpu=gpu_options(precision=1, seed=seed ^ 0xABCDEF, use_surrogate=1))
    pilot.share_surrogate(sur)
    r, t = pilot.sample_event_points(share=min(1.0, 4e5 / n_hist), max_points=1 << 14)
    held_out = sur.validate_surrogate(r, t, hits=1 << 24)
    pilot.close()

    def runner(sim):
        def step():
            out = sim.msim()
            tm = sim.timing()
            if sim in last:
                sim.free_raw(last[sim])
            last[sim] = out
            return tm
        return step

    last = {}
    tms_g, wall_g, _ = timed_steps(args, runner(grid_run), local)
    tms, wall, clocks = timed_steps(args, runner(sur), local)
    ksum = sum(t["kernel_ms"] for t in tms)
    ksum_g = sum(t["kernel_ms"] for t in tms_g)
    out_s, out_g = last[sur], last[grid_run]
    # all-FP64 grid run of the same photons: the precision reference
    ref = Simulation(spec, options=options, gpu=g64)
    ref.set_solid_angle(ax["r"], ax["theta"], ax["grid"])
    out_64 = ref.msim()
    errs = {"vs_grid_fp32": line_error(out_s, out_g, floor=1e-3), "vs_grid_fp64": line_error(out_s, out_64, 1e-3),
            "grid_fp32_vs_grid_fp64": line_error(out_g, out_64, floor=1e-3),
            "lines": "lines with >= 0.1% of the strongest, summed over orders; same photon streams"}
    for o, sm in ((out_s, sur), (out_g, grid_run), (out_64, ref)):
        sm.free_raw(o)
    ref.close()
    gsim.close()
    step_s, step_g = wall / args.steps, wall_g / args.steps
    extra = {"grid": "1000 x 1000, FP64 integrator, %d samples per point" % 5000, "grid_s": grid_s,
             "surrogate": dict(rep, n_train=args.n_train_surrogate, hits_train=args.hits_train,
                               epochs=args.epochs_surrogate,
                               tolerance=args.tolerance, hits_check=args.hits_check, wall_s=train_s,
                               sampling="uniform over the sample volume (2 cm around the beam axis)"
                               if args.surrogate_points == "volume" else
                               "the estimator's query points of a pilot run (another seed)"),
             "held_out": held_out,
             "l2": "tables and grid above 129 MB: no; inputs smaller than L2, no flush between steps"}
    line = {"metric": PLAIN_METRIC + " (surrogate-served transport)", "value": n_hist * args.steps / (ksum / 1e3),
            "unit": "histories/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ksum / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 transport, f64 tallies", "data": "synthetic (config-1 sample, 17.44 keV line)",
            "config": workload_config(args, extra),
            "gpu_launches": sum(t["launches"] for t in tms),
            "phases_ms_per_step": {k: statistics.mean(t[k + "_ms"] for t in tms)
                                   for k in ("transport", "sort", "surrogate", "estimator")},
            "events_per_step": statistics.mean(t["events"] for t in tms),
            "surrogate_fallbacks_per_step": statistics.mean(t["surrogate_fallbacks"] for t in tms),
            "e2e": {"value": n_hist * args.steps / wall, "unit": "histories/s",
                    "h2d_bytes_per_step": int(statistics.mean(t["h2d_bytes"] for t in tms)),
                    "d2h_bytes_per_step": int(statistics.mean(t["d2h_bytes"] for t in tms))},
            "grid_path": {"value": n_hist * args.steps / (ksum_g / 1e3), "e2e": n_hist * args.steps / wall_g,
                          "phases_ms_per_step": dict({k: statistics.mean(t[k + "_ms"] for t in tms_g)
                                                      for k in ("transport", "sort", "estimator")},
                                                     off_grid_solid_angles=statistics.mean(t["surrogate_ms"]
                                                                                           for t in tms_g)),
                          "job_s": grid_s + step_g, "job": "grid + one step"},
            "surrogate_path_job_s": train_s + step_s,
            "line_error": errs,
            "clocks": clocks}
    if cudart is not None:
        cudart.cudaDeviceSynchronize()
    return line, [grid_run, sur], [spec], options


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        cudart = load_cudart()
        if cudart is not None:
            cudart.cudaSetDevice(local)
    from xmimsim_gb300.build import build_all
    build_all()
    arm = {"batched": batched_arm, "plain": plain_arm, "surrogate": surrogate_arm,
           "precision": precision_arm}[args.workload]
    line, sims, specs, options = arm(args, ws, rank, local)
    if ws > 1:
        # whole job: the histories of every rank over the slowest rank's time
        # (device time for value, host wall for e2e)
        import torch
        n_step = line["value"] * line["ms_per_step"] / 1e3  # this rank's histories per step
        e2e_s = n_step / line["e2e"]["value"] if line.get("e2e") else 0.0
        t = torch.tensor([line["ms_per_step"], e2e_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        n = torch.tensor([n_step], dtype=torch.float64, device="cuda")
        dist.all_reduce(n, op=dist.ReduceOp.SUM)
        line["ms_per_step"] = t[0].item()
        line["value"] = n.item() / (line["ms_per_step"] / 1e3)
        if line.get("e2e") and t[1].item() > 0:
            line["e2e"]["value"] = n.item() / t[1].item()
    if rank == 0 and not args.no_cpu_baseline:
        cspecs, coptions, what = cpu_sample_specs(args, rank)
        cv, cn, cdt, words_tr, words_est = run_cpu_sample(cspecs, coptions, args.cpu_sample, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": cv, "unit": "histories/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d photons (%.2f s) over %s" % (cn, cdt, what)}
        word = 4 if line["dtype"].startswith("f32") else 8
        qev = line["config"].get("autotuned", {}).get("queue_events") or (1 << 25)
        n_int = 6 if args.workload == "plain" else 4
        per_launch = min(qev // n_int, line["config"]["photons_per_step"])
        tph = ESTIMATOR_DRAM_BYTES_PER_HISTORY.get(args.workload) if word == 4 else None
        line["roofline"] = roofline_block(line["phases_ms_per_step"], line["config"]["photons_per_step"],
                                          words_tr, words_est, word, tph, per_launch)
    if rank == 0:
        print(json.dumps(line))
    for s in sims:
        s.close()
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
