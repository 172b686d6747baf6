#!/usr/bin/env python3
"""Benchmark: photon histories/s of the XRF transport on GB300.

Workload (default): the production-size plain configuration -- 5 random
layers (seed 2) of 3-12 elements, Rh tube at 40 kV behind 125 um Be in 400
intervals plus the Rh K/L lines, 1e8 photons per step, 6 interactions,
variance reduction on, all-FP64 transport (``--precision fp32`` for the FP32
transport / FP64 tallies variant).

One step = one xmi_main_msim call over the full photon budget.
  value  -- histories / kernel time (CUDA events on the launching stream;
            tables and solid-angle grid resident on the device),
  e2e    -- histories / wall time of the public C-ABI call from the host
            (source items uploaded, tallies copied back and reshaped into the
            reference's output layouts inside the timed region).
Multi-GPU (torchrun): every rank simulates its own disjoint photon range of
the same size (weak scaling, no data-path collective); the tallies are summed
over ranks with one reduce after the timed region.

``--impl reference`` times the reference algorithm's CPU path: the FP64 C
restatement under oracle/ (the reference's Fortran build needs gfortran and
xraylib, absent here) with all host threads, each step a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--photons", type=float, default=1e8, help="photons per step (per GPU)")
    p.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    p.add_argument("--cpu-sample", type=int, default=200000, help="photons of the CPU-baseline sample")
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


def workload_spec(photons: int):
    from xmimsim_gb300 import configs
    return configs.config2(total_photons=int(photons)), dict(configs.C2_OPTIONS, use_sum_peaks=0)


def run_cpu_sample(spec, options, n_sample: int, threads: int):
    """Times the FP64 CPU restatement (all threads) on a bounded sample of the
    workload; returns (histories/s, histories, seconds, words/history)."""
    from oracle import oracle_api
    from xmimsim_gb300 import Simulation, gpu_options
    import numpy as np
    n_items = len(spec.discrete) + max(0, len(spec.continuous) - 1)
    per_item = max(1, n_sample // max(1, n_items))
    sim = Simulation(spec, options=options, gpu=gpu_options(seed=0x5EED0001))
    # the CPU path uses a coarse grid over the same axes, built here (untimed) so that no GPU is needed
    r, t = sim.grid_axes(64, 64)
    sim.set_solid_angle(r, t, np.zeros((64, 64)))
    sim.prepare()
    g = oracle_api.solid_angle_points(sim.bundle_ptr(), r, t, 0, 64 * 64, 500).reshape(64, 64)
    sim.set_solid_angle(r, t, g)
    sim.prepare()
    oracle_api.words_counted_split()
    t0 = time.perf_counter()
    oracle_api.msim(sim.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels, threads=threads,
                    max_photons_per_item=per_item)
    dt = time.perf_counter() - t0
    words, words_est = oracle_api.words_counted_split()
    n = per_item * n_items
    sim.close()
    return n / dt, n, dt, (words - words_est) / n, words_est / n


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from xmimsim_gb300 import Simulation
    spec, options = workload_spec(args.photons)
    threads = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        v, n, dt, _, _ = run_cpu_sample(spec, options, args.cpu_sample, threads)
        if i >= args.warmup:
            vals.append((v, n, dt))
    value = statistics.median(v for v, _, _ in vals)
    sample = "%d photons per step of the %.0e-photon workload" % (vals[0][1], args.photons)
    line = {"metric": "photon histories/s", "value": value, "unit": "histories/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(d for _, _, d in vals) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random 5-layer sample, Rh tube spectrum)",
            "config": {"workload": "plain 5-layer Rh 40 kV, 6 interactions, VR on", "photons_per_step": vals[0][1]},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    ws, rank, local = dist_env()
    import ctypes as C
    import numpy as np
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from xmimsim_gb300 import Simulation, abi, gpu_options
    from xmimsim_gb300.build import build_all
    build_all()
    lib = abi.load()
    cudart = None
    try:
        cudart = C.CDLL("libcudart.so")
    except OSError:
        import glob
        c = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        cudart = C.CDLL(c[0]) if c else None
    if cudart is not None and ws > 1:
        cudart.cudaSetDevice(local)

    spec, options = workload_spec(args.photons)
    precision = 0 if args.precision == "fp64" else 1
    t_setup = time.perf_counter()
    sim = Simulation(spec, options=options, gpu=gpu_options(precision=precision, seed=0x5EED0001 + rank))
    sim.solid_angle()
    t_setup = time.perf_counter() - t_setup
    n_hist = int(spec.n_photons_interval) * (len(spec.continuous) - 1) + int(spec.n_photons_line) * len(spec.discrete)

    def step():
        out = sim.msim()
        tm = sim.timing()
        sim.free_raw(out)
        return out, tm

    for _ in range(args.warmup):
        step()
    if ws > 1:
        dist.barrier()
    if cudart is not None:
        cudart.cudaDeviceSynchronize()
    kernel_ms, launches, phases = [], 0, []
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out, tm = step()
            kernel_ms.append(tm["kernel_ms"])
            launches += tm["launches"]
            phases.append(tm)
        if cudart is not None:
            cudart.cudaDeviceSynchronize()
        wall = time.perf_counter() - t0
    if ws > 1:
        import torch
        t = torch.tensor([wall, sum(kernel_ms)], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        wall, ksum = t.tolist()
        # the reference's MPI reduce of the tallies (bin/xmimsim.c:402-410), after the timed region
        ch = torch.tensor(out["channels"], device="cuda")
        dist.all_reduce(ch)
    else:
        ksum = sum(kernel_ms)
    total_hist = n_hist * ws * args.steps
    value = total_hist / (ksum / 1e3)
    e2e = total_hist / wall
    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return
    line = {"metric": "photon histories/s", "value": value, "unit": "histories/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ksum / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if precision == 0 else "f32 transport, f64 tallies",
            "data": "synthetic (seeded random 5-layer sample, Rh tube spectrum)",
            "config": {"workload": "plain 5-layer Rh 40 kV, 400 intervals + Rh K/L lines, 6 interactions, VR on",
                       "photons_per_step": n_hist, "elements": sum(len(l.Z) for l in spec.layers),
                       "l2": "inputs larger than L2 (angular tables of all elements exceed 129 MB)",
                       "solid_angle_grid_s": t_setup},
            "gpu_launches": launches,
            "phases_ms_per_step": {k: statistics.mean(p[k + "_ms"] for p in phases)
                                   for k in ("transport", "sort", "estimator")},
            "events_per_step": statistics.mean(p["events"] for p in phases),
            "e2e": {"value": e2e, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "clocks": clocks.summary()}
    # host<->device bytes of one public call: source items in, tallies out
    n_items = (len(spec.continuous) - 1) + len(spec.discrete)
    line["e2e"]["h2d_bytes_per_step"] = n_items * (128 + 8)
    nslots = 0
    line["e2e"]["d2h_bytes_per_step"] = int(8 * (spec.n_interactions_trajectory + 1) * spec.nchannels)
    if not args.no_cpu_baseline:
        cv, cn, cdt, words_tr, words_est = run_cpu_sample(spec, options, args.cpu_sample, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": cv, "unit": "histories/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d photons (%.2f s) of the same workload" % (cn, cdt)}
        # dominant kernel: algorithmic table bytes it reads per history (counted
        # by the instrumented oracle on the sample) over its device time
        word = 8 if precision == 0 else 4
        ph = line["phases_ms_per_step"]
        kern = "estimator_kernel" if ph["estimator"] >= ph["transport"] else "transport_kernel"
        kms = ph["estimator"] if kern == "estimator_kernel" else ph["transport"]
        bph = (words_est if kern == "estimator_kernel" else words_tr) * word
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = bph * n_hist / (kms / 1e3) / 1e9 if kms > 0 else 0.0
        line["roofline"] = {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": None,
                            "algorithmic_bytes_per_history": bph,
                            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback 6.8 TB/s"}
    print(json.dumps(line))
    sim.close()
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
