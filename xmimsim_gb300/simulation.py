"""Python host mirror of the reference's simulation call chain.

``Simulation`` follows bin/xmimsim.c:249-669 / tests/libxmimsim-test.c:182-270:
xmi_input_C2F -> xmi_init_input -> xmi_init_from_hdf5 -> xmi_solid_angle_calculation
-> xmi_main_msim -> xmi_escape_ratios_calculation -> xmi_detector_convolute_all,
every step a call into libxmimsim_gb300.so.  Outputs come back as numpy
arrays in the reference's layouts.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import abi


@dataclass
class Layer:
    Z: Sequence[int]
    weight: Sequence[float]
    density: float
    thickness: float


@dataclass
class DiscreteLine:
    energy: float
    horizontal_intensity: float
    vertical_intensity: float
    sigma_x: float = 0.0
    sigma_xp: float = 0.0
    sigma_y: float = 0.0
    sigma_yp: float = 0.0
    distribution_type: int = 0
    scale_parameter: float = 0.0


@dataclass
class ContinuousPoint:
    energy: float
    horizontal_intensity: float
    vertical_intensity: float
    sigma_x: float = 0.0
    sigma_xp: float = 0.0
    sigma_y: float = 0.0
    sigma_yp: float = 0.0


@dataclass
class InputSpec:
    """Python description of an ``xmi_input`` (defaults of xmi_input_init_empty)."""
    layers: list[Layer]
    reference_layer: int = 1
    n_photons_interval: int = 10000
    n_photons_line: int = 100000
    n_interactions_trajectory: int = 4
    d_sample_source: float = 100.0
    n_sample_orientation: tuple = (0.0, -(2.0 ** 0.5) / 2.0, (2.0 ** 0.5) / 2.0)
    p_detector_window: tuple = (0.0, 1.0, 100.0)
    n_detector_orientation: tuple = (0.0, -1.0, 0.0)
    area_detector: float = 0.3
    collimator_height: float = 0.0
    collimator_diameter: float = 0.0
    d_source_slit: float = 100.0
    slit_size_x: float = 0.001
    slit_size_y: float = 0.001
    discrete: list[DiscreteLine] = field(default_factory=lambda: [DiscreteLine(28.0, 1e12, 1e9)])
    continuous: list[ContinuousPoint] = field(default_factory=list)
    exc_layers: list[Layer] = field(default_factory=list)
    det_layers: list[Layer] = field(default_factory=lambda: [Layer([4], [1.0], 1.85, 0.002)])
    detector_type: int = 0
    live_time: float = 1.0
    pulse_width: float = 10e-6
    gain: float = 0.02
    zero: float = 0.0
    fano: float = 0.12
    noise: float = 0.1
    nchannels: int = 2048
    crystal_layers: list[Layer] = field(default_factory=lambda: [Layer([14], [1.0], 2.33, 0.5)])

    def to_c(self) -> "CInput":
        return CInput(self)


class CInput:
    """ctypes ``xmi_input`` built from an InputSpec; keeps every buffer alive."""

    def __init__(self, s: InputSpec):
        self._keep = []
        g = abi.XmiGeneral(8.1, b"", s.n_photons_interval, s.n_photons_line, s.n_interactions_trajectory, b"")
        comp = abi.XmiComposition(len(s.layers), self._layers(s.layers), s.reference_layer)
        geo = abi.XmiGeometry(s.d_sample_source, (C.c_double * 3)(*s.n_sample_orientation),
                              (C.c_double * 3)(*s.p_detector_window), (C.c_double * 3)(*s.n_detector_orientation),
                              s.area_detector, s.collimator_height, s.collimator_diameter, s.d_source_slit,
                              s.slit_size_x, s.slit_size_y)
        disc = (abi.XmiEnergyDiscrete * max(1, len(s.discrete)))(
            *[abi.XmiEnergyDiscrete(d.energy, d.horizontal_intensity, d.vertical_intensity, d.sigma_x, d.sigma_xp,
                                    d.sigma_y, d.sigma_yp, d.distribution_type, d.scale_parameter)
              for d in s.discrete])
        cont = (abi.XmiEnergyContinuous * max(1, len(s.continuous)))(
            *[abi.XmiEnergyContinuous(c.energy, c.horizontal_intensity, c.vertical_intensity, c.sigma_x, c.sigma_xp,
                                      c.sigma_y, c.sigma_yp) for c in s.continuous])
        self._keep += [disc, cont]
        exc = abi.XmiExcitation(len(s.discrete), C.cast(disc, C.POINTER(abi.XmiEnergyDiscrete)),
                                len(s.continuous), C.cast(cont, C.POINTER(abi.XmiEnergyContinuous)))
        absb = abi.XmiAbsorbers(len(s.exc_layers), self._layers(s.exc_layers), len(s.det_layers),
                                self._layers(s.det_layers))
        det = abi.XmiDetector(s.detector_type, s.live_time, s.pulse_width, s.gain, s.zero, s.fano, s.noise,
                              s.nchannels, len(s.crystal_layers), self._layers(s.crystal_layers))
        parts = [g, comp, geo, exc, absb, det]
        self._keep += parts
        self.input = abi.XmiInput(*[C.pointer(p) for p in parts])

    def _layers(self, layers: list[Layer]):
        arr = (abi.XmiLayer * max(1, len(layers)))()
        for i, l in enumerate(layers):
            z = (C.c_int * len(l.Z))(*l.Z)
            w = (C.c_double * len(l.weight))(*l.weight)
            self._keep += [z, w]
            arr[i] = abi.XmiLayer(len(l.Z), C.cast(z, abi.c_int_p), C.cast(w, abi.c_double_p), l.density, l.thickness)
        self._keep.append(arr)
        return C.cast(arr, C.POINTER(abi.XmiLayer))


def make_options(**kw) -> abi.XmiMainOptions:
    lib = abi.load()
    p = lib.xmi_main_options_new()
    opts = abi.XmiMainOptions()
    C.pointer(opts)[0] = p.contents
    lib.xmi_main_options_free(p)
    for k, v in kw.items():
        if not hasattr(opts, k):
            raise KeyError(k)
        setattr(opts, k, v)
    return opts


def gpu_options(precision: int = 0, seed: int = 0, threads_per_block: int = 0, blocks_per_sm: int = 0,
                use_surrogate: int = 0, surrogate_tolerance: float = 1e-3,
                solid_angle_stream: int = 0, grid_n: int = 0, overlap_chunks: int = 0,
                estimator_blocks_per_sm: int = 0) -> abi.XmiGpuOptions:
    """grid_n: points of the solid-angle grid along r and along theta (0: the
    reference's 1024).  overlap_chunks=1 runs the next chunk's transport
    beside the current chunk's sort, solid angles and estimator (two event
    queues) instead of one after another; estimator_blocks_per_sm caps the
    estimator's resident blocks per SM (0: as many as fit)."""
    g = abi.XmiGpuOptions()
    abi.load().xmi_gpu_default_options(C.byref(g))
    g.precision, g.seed, g.solid_angle_stream = precision, seed, solid_angle_stream
    g.threads_per_block, g.blocks_per_sm = threads_per_block, blocks_per_sm
    g.use_surrogate, g.surrogate_tolerance = use_surrogate, surrogate_tolerance
    g.grid_nr = g.grid_nt = grid_n
    g.overlap_chunks, g.estimator_blocks_per_sm = overlap_chunks, estimator_blocks_per_sm
    return g


class XmiError(RuntimeError):
    pass


def _check(rv: int, what: str) -> None:
    if rv != 1:
        raise XmiError(f"{what} failed: {abi.last_error()}")


def last_timing() -> dict:
    """Device and wall times, phases, surrogate counters and host<->device
    bytes of the calling thread's last xmi_main_msim / xmi_main_msim_batch."""
    lib = abi.load()
    t, tot, n = C.c_double(), C.c_double(), C.c_int()
    lib.xmi_gpu_last_timing(C.byref(t), C.byref(tot), C.byref(n))
    out = {"kernel_ms": t.value, "total_ms": tot.value, "launches": n.value}
    tr, so, es, ev = C.c_double(), C.c_double(), C.c_double(), C.c_longlong()
    lib.xmi_gpu_last_phases(C.byref(tr), C.byref(so), C.byref(es), C.byref(ev))
    out.update(transport_ms=tr.value, sort_ms=so.value, estimator_ms=es.value, events=ev.value)
    sg, fb = C.c_double(), C.c_longlong()
    lib.xmi_gpu_last_surrogate(C.byref(sg), C.byref(fb))
    out.update(surrogate_ms=sg.value, surrogate_fallbacks=fb.value)
    hd, dh = C.c_longlong(), C.c_longlong()
    lib.xmi_gpu_last_transfers(C.byref(hd), C.byref(dh))
    out.update(h2d_bytes=hd.value, d2h_bytes=dh.value)
    gu = C.c_int()
    lib.xmi_gpu_last_graph(C.byref(gu))
    out.update(graph_updated=gu.value)
    return out


class Simulation:
    """One simulation set-up: input handle + table bundle (no GPU work yet)."""

    def __init__(self, spec: InputSpec, options: dict | None = None, gpu: abi.XmiGpuOptions | None = None):
        self.lib = abi.load()
        self.spec = spec
        self.cinput = spec.to_c()
        self.options = make_options(**(options or {}))
        self.inputF = C.c_void_p()
        self.tables = C.c_void_p()
        _check(self.lib.xmi_input_C2F(C.byref(self.cinput.input), C.byref(self.inputF)), "xmi_input_C2F")
        _check(self.lib.xmi_init_input(C.byref(self.inputF)), "xmi_init_input")
        self.gpu = gpu if gpu is not None else gpu_options()
        if gpu is not None:
            _check(self.lib.xmi_gpu_set_options(self.inputF, C.byref(gpu)), "xmi_gpu_set_options")
        _check(self.lib.xmi_init_from_hdf5(None, self.inputF, C.byref(self.tables), C.byref(self.options)),
               "xmi_init_from_hdf5")
        _check(self.lib.xmi_update_input_from_hdf5(self.inputF, self.tables), "xmi_update_input_from_hdf5")
        self._sa = None

    # -- solid angle -------------------------------------------------------
    def solid_angle(self) -> C.POINTER(abi.XmiSolidAngle):
        if self._sa is None:
            p = C.POINTER(abi.XmiSolidAngle)()
            _check(self.lib.xmi_solid_angle_calculation_cuda(self.inputF, C.byref(p), None, C.byref(self.options)),
                   "xmi_solid_angle_calculation_cuda")
            self._sa = p
            self._sa_owned = True
        return self._sa

    def solid_angle_grid(self) -> dict:
        sa = self.solid_angle().contents
        nr, nt = sa.grid_dims_r_n, sa.grid_dims_theta_n
        return {"r": np.ctypeslib.as_array(sa.grid_dims_r_vals, (nr,)).copy(),
                "theta": np.ctypeslib.as_array(sa.grid_dims_theta_vals, (nt,)).copy(),
                "grid": np.ctypeslib.as_array(sa.solid_angles, (nt, nr)).copy()}

    def grid_axes(self, nr: int = 1024, nt: int = 1024):
        """The (r, theta) axes xmi_solid_angle_calculation uses (xmi_solid_angle_inputs_f)."""
        r = np.zeros(nr)
        t = np.zeros(nt)
        f = self.lib.xmi_solid_angle_axes
        f.restype = None
        f.argtypes = [C.c_void_p, C.c_int, C.c_int, abi.c_double_p, abi.c_double_p]
        f(self.inputF, nr, nt, r.ctypes.data_as(abi.c_double_p), t.ctypes.data_as(abi.c_double_p))
        return r, t

    def set_solid_angle(self, r: np.ndarray, theta: np.ndarray, grid: np.ndarray) -> None:
        """Uses a caller-supplied solid-angle grid ([theta][r]) instead of computing one."""
        self._sa_keep = [np.ascontiguousarray(r, dtype=np.float64), np.ascontiguousarray(theta, dtype=np.float64),
                         np.ascontiguousarray(grid, dtype=np.float64)]
        sa = abi.XmiSolidAngle(self._sa_keep[2].ctypes.data_as(abi.c_double_p), len(r), len(theta),
                               self._sa_keep[0].ctypes.data_as(abi.c_double_p),
                               self._sa_keep[1].ctypes.data_as(abi.c_double_p), None)
        self._sa_struct = sa
        self._sa = C.pointer(sa)
        self._sa_owned = False

    def set_gpu(self, gpu: abi.XmiGpuOptions) -> None:
        _check(self.lib.xmi_gpu_set_options(self.inputF, C.byref(gpu)), "xmi_gpu_set_options")
        self.gpu = gpu

    # -- transport -----------------------------------------------------------
    def surrogate_on(self) -> bool:
        rep = np.zeros(6)
        return bool(self.gpu.use_surrogate) and \
            self.lib.xmi_gpu_surrogate_report(self.inputF, rep.ctypes.data_as(abi.c_double_p)) == 1

    def prepare(self, n_mpi_hosts: int = 1) -> None:
        """Builds the run part of the bundle exactly as xmi_main_msim does (no GPU)."""
        sa = self._sa if self.options.use_variance_reduction else None
        _check(self.lib.xmi_gpu_prepare_run(self.inputF, self.tables, C.byref(self.options), n_mpi_hosts, sa),
               "xmi_gpu_prepare_run")

    def set_replica(self, replica: int, n_replicas: int) -> None:
        """This process simulates photons [r*n/R, (r+1)*n/R) of every source item."""
        _check(self.lib.xmi_gpu_set_replica(self.tables, replica, n_replicas), "xmi_gpu_set_replica")

    def bundle_ptr(self) -> int:
        return self.lib.xmi_gpu_bundle(self.tables)

    def msim(self, n_mpi_hosts: int = 1) -> dict:
        N = self.spec.n_interactions_trajectory
        nch = self.spec.nchannels
        ch = abi.c_double_p()
        br = abi.c_double_p()
        vr = abi.c_double_p()
        sa = self.solid_angle() if self.options.use_variance_reduction and not self.surrogate_on() else None
        _check(self.lib.xmi_main_msim(self.inputF, self.tables, n_mpi_hosts, C.byref(ch), C.byref(self.options),
                                      C.byref(br), C.byref(vr), sa), "xmi_main_msim")
        out = {"channels": np.ctypeslib.as_array(ch, ((N + 1), nch)).copy(),
               "brute": np.ctypeslib.as_array(br, (100, 385, N)).copy(),
               "var_red": np.ctypeslib.as_array(vr, (100, 385, N)).copy() if vr else None,
               "raw": (ch, br, vr)}
        return out

    @staticmethod
    def msim_batch(sims: "Sequence[Simulation]", copy: bool = True) -> list[dict]:
        """Runs several configurations in one batched launch sequence
        (xmi_main_msim_batch); one output dict per configuration, as msim().
        copy=False returns views of the library's output arrays instead of
        copies (no host copy of the dense reference layouts); they stay valid
        until free_raw releases them."""
        lib = abi.load()
        n = len(sims)
        ins = (C.c_void_p * n)(*[s.inputF.value for s in sims])
        tabs = (C.c_void_p * n)(*[s.tables.value for s in sims])
        opts = (C.POINTER(abi.XmiMainOptions) * n)(*[C.pointer(s.options) for s in sims])
        sas = (C.POINTER(abi.XmiSolidAngle) * n)(
            *[s.solid_angle() if s.options.use_variance_reduction and not s.surrogate_on()
              else C.POINTER(abi.XmiSolidAngle)() for s in sims])
        ch = (abi.c_double_p * n)()
        br = (abi.c_double_p * n)()
        vr = (abi.c_double_p * n)()
        _check(lib.xmi_main_msim_batch(n, ins, tabs, opts, sas, ch, br, vr), "xmi_main_msim_batch")
        outs = []
        cp = (lambda a: a.copy()) if copy else (lambda a: a)
        for i, s in enumerate(sims):
            N = s.spec.n_interactions_trajectory
            nch = s.spec.nchannels
            outs.append({"channels": cp(np.ctypeslib.as_array(ch[i], ((N + 1), nch))),
                         "brute": cp(np.ctypeslib.as_array(br[i], (100, 385, N))),
                         "var_red": cp(np.ctypeslib.as_array(vr[i], (100, 385, N))) if vr[i] else None,
                         "raw": (ch[i], br[i], vr[i])})
        return outs

    @staticmethod
    def autotune_batch(sims: "Sequence[Simulation]", share: float = 1.0 / 64) -> dict:
        """Picks the wavefront launch shape and the estimator queue size of a
        batch by timing short batched runs (xmi_gpu_autotune_batch) and keeps
        them in every configuration's GPU options."""
        lib = abi.load()
        n = len(sims)
        ins = (C.c_void_p * n)(*[s.inputF.value for s in sims])
        tabs = (C.c_void_p * n)(*[s.tables.value for s in sims])
        opts = (C.POINTER(abi.XmiMainOptions) * n)(*[C.pointer(s.options) for s in sims])
        sas = (C.POINTER(abi.XmiSolidAngle) * n)(
            *[s.solid_angle() if s.options.use_variance_reduction and not s.surrogate_on()
              else C.POINTER(abi.XmiSolidAngle)() for s in sims])
        rep = np.zeros(4)
        _check(lib.xmi_gpu_autotune_batch(n, ins, tabs, opts, sas, share, rep.ctypes.data_as(abi.c_double_p)),
               "xmi_gpu_autotune_batch")
        for s in sims:
            s.gpu.threads_per_block, s.gpu.blocks_per_sm, s.gpu.queue_events = int(rep[0]), int(rep[1]), int(rep[2])
        return {"threads_per_block": int(rep[0]), "blocks_per_sm": int(rep[1]), "queue_events": int(rep[2]),
                "best_trial_ms": float(rep[3]), "share": share}

    def build_surrogate(self, n_train: int = 1 << 21, hits_train: int = 2048, epochs: int = 8,
                        hits_check: int = 1 << 20) -> dict:
        """Trains the solid-angle surrogate network (xmi_gpu_build_surrogate)."""
        rep = np.zeros(6)
        _check(self.lib.xmi_gpu_build_surrogate(self.inputF, n_train, hits_train, epochs, hits_check,
                                                rep.ctypes.data_as(abi.c_double_p)), "xmi_gpu_build_surrogate")
        keys = ("median_rel_err", "max_rel_err_kept", "flagged_fraction", "train_loss", "seconds", "cells")
        return dict(zip(keys, rep.tolist()))

    def sample_event_points(self, share: float, max_points: int) -> tuple[np.ndarray, np.ndarray]:
        """(r, theta) of about max_points solid-angle queries of the estimator
        in a pilot run over `share` of the photons (xmi_gpu_sample_event_points)."""
        r = np.zeros(max_points)
        t = np.zeros(max_points)
        n = C.c_int(0)
        _check(self.lib.xmi_gpu_sample_event_points(self.inputF, self.tables, C.byref(self.options), share,
                                                    max_points, r.ctypes.data_as(abi.c_double_p),
                                                    t.ctypes.data_as(abi.c_double_p), C.byref(n)),
               "xmi_gpu_sample_event_points")
        return r[:n.value].copy(), t[:n.value].copy()

    def build_surrogate_points(self, r: np.ndarray, theta: np.ndarray, hits_train: int = 1024, epochs: int = 8,
                               hits_check: int = 1 << 20) -> dict:
        """Trains the surrogate on the given (r, theta) points (xmi_gpu_build_surrogate_points)."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        rep = np.zeros(6)
        _check(self.lib.xmi_gpu_build_surrogate_points(self.inputF, len(r), r.ctypes.data_as(abi.c_double_p),
                                                       theta.ctypes.data_as(abi.c_double_p), hits_train, epochs,
                                                       hits_check, rep.ctypes.data_as(abi.c_double_p)),
               "xmi_gpu_build_surrogate_points")
        keys = ("median_rel_err", "max_rel_err_kept", "flagged_fraction", "train_loss", "seconds", "cells")
        return dict(zip(keys, rep.tolist()))

    def surrogate_eval(self, r: np.ndarray, theta: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """(omega, source) the transport would take from the trained surrogate
        at these points: source 0 network, 1 tabulated integrator of a flagged
        cell, 2 outside the checked region (integrated per event; omega -1),
        3 below the lowest theta (omega 0) -- xmi_gpu_surrogate_eval."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        om = np.zeros(len(r))
        src = np.zeros(len(r), dtype=np.int32)
        _check(self.lib.xmi_gpu_surrogate_eval(self.inputF, len(r), r.ctypes.data_as(abi.c_double_p),
                                               theta.ctypes.data_as(abi.c_double_p), om.ctypes.data_as(abi.c_double_p),
                                               src.ctypes.data_as(C.POINTER(C.c_int))), "xmi_gpu_surrogate_eval")
        return om, src

    def solid_angle_points(self, r: np.ndarray, theta: np.ndarray, hits: int, precision: int = 0,
                           seed: int = 0x5EED0007) -> np.ndarray:
        """The engine's solid-angle integrator at arbitrary (r, theta) points,
        `hits` cone samples each (xmi_gpu_solid_angle_points)."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        om = np.zeros(len(r))
        _check(self.lib.xmi_gpu_solid_angle_points(self.inputF, len(r), r.ctypes.data_as(abi.c_double_p),
                                                   theta.ctypes.data_as(abi.c_double_p), hits, precision, seed,
                                                   om.ctypes.data_as(abi.c_double_p)), "xmi_gpu_solid_angle_points")
        return om

    def validate_surrogate(self, r: np.ndarray, theta: np.ndarray, hits: int = 1 << 24,
                           seed: int = 0x5EED0077) -> dict:
        """Held-out check of the trained surrogate at points it was not
        trained or checked on: the solid angle the transport would take
        (surrogate_eval) against the integrator with `hits` samples per point
        (FP32; its relative noise is sqrt((1 - p) / (p hits)) for a hit share
        p).  Per source: points, median / RMS / 99th-percentile relative
        error and the mean (bias)."""
        om, src = self.surrogate_eval(r, theta)
        truth = self.solid_angle_points(r, theta, hits=hits, precision=1, seed=seed)
        out = {"points": int(len(r)), "hits": hits,
               "share": {name: float((src == k).mean()) for k, name in
                         enumerate(("network", "table", "integrator", "zero"))}}
        for k, name in ((0, "network"), (1, "table")):
            m = (src == k) & (truth > 0)
            if m.any():
                e = (om[m] - truth[m]) / truth[m]
                out[name] = {"points": int(m.sum()), "median": float(np.median(np.abs(e))),
                             "rms": float(np.sqrt((e ** 2).mean())), "p99": float(np.quantile(np.abs(e), 0.99)),
                             "bias": float(e.mean())}
        return out

    def share_surrogate(self, other: "Simulation") -> None:
        """Serves this configuration's solid angles from the network trained
        for `other` (same detector and collimator; xmi_gpu_share_surrogate)."""
        _check(self.lib.xmi_gpu_share_surrogate(other.inputF, self.inputF), "xmi_gpu_share_surrogate")

    def free_raw(self, out: dict) -> None:
        for p in out.pop("raw", ()):
            if p:
                self.lib.xmi_free(C.cast(p, C.c_void_p))

    def timing(self) -> dict:
        return last_timing()

    # -- detector response -------------------------------------------------
    def escape_ratios(self, n_photons: int | None = None, n_input_energies: int | None = None):
        ero = self.lib.xmi_get_default_escape_ratios_options()
        if n_photons is not None:
            ero.n_photons = n_photons
        if n_input_energies is not None:
            ero.n_input_energies = n_input_energies
        p = C.POINTER(abi.XmiEscapeRatios)()
        self.lib.xmi_escape_ratios_calculation(C.byref(self.cinput.input), C.byref(p), None, None,
                                               C.byref(self.options), ero)
        if not p:
            raise XmiError("xmi_escape_ratios_calculation failed: " + abi.last_error())
        return p

    def convolute(self, channels: np.ndarray, escape=None, zero_interaction: int = 0) -> np.ndarray:
        N = channels.shape[0] - 1
        nch = channels.shape[1]
        rows = [np.ascontiguousarray(channels[i], dtype=np.float64) for i in range(N + 1)]
        noconv = (abi.c_double_p * (N + 1))(*[r.ctypes.data_as(abi.c_double_p) for r in rows])
        conv = (abi.c_double_p * (N + 1))()
        self.lib.xmi_detector_convolute_all(self.inputF, noconv, conv, None, None, C.byref(self.options),
                                            escape, N, zero_interaction)
        out = np.zeros((N + 1, nch))
        start = 0 if zero_interaction else 1
        for i in range(start, N + 1):
            if not conv[i]:
                raise XmiError("xmi_detector_convolute_all failed: " + abi.last_error())
            out[i] = np.ctypeslib.as_array(conv[i], (nch,))
            self.lib.xmi_free(C.cast(conv[i], C.c_void_p))
        return out

    def close(self) -> None:
        if self._sa is not None:
            if getattr(self, "_sa_owned", False):
                self.lib.xmi_free_solid_angle(self._sa)
            self._sa = None
        if self.tables:
            self.lib.xmi_free_hdf5_F(C.byref(self.tables))
        if self.inputF:
            self.lib.xmi_free_input_F(C.byref(self.inputF))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
