"""TEST INFRASTRUCTURE: ctypes access to the FP64 CPU oracle (oracle/*.c).

Only the test-suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline use this module, always as the checker or the timed CPU baseline,
never inside the engine.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_build" / "liboracle_xmimsim.so"
_lib = None


class OracleEscape(C.Structure):
    _fields_ = [("n_el", C.c_int), ("nfe", C.c_int), ("nce", C.c_int), ("nco", C.c_int),
                ("edge", C.POINTER(C.c_double)), ("line_e", C.POINTER(C.c_double)),
                ("fluo", C.POINTER(C.c_double)), ("fe", C.POINTER(C.c_double)),
                ("comp", C.POINTER(C.c_double)), ("ce", C.POINTER(C.c_double)), ("co", C.POINTER(C.c_double))]


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing: run __graft_entry__.build()")
        _lib = C.CDLL(str(LIB))
        dp = C.POINTER(C.c_double)
        _lib.oracle_xmi_main_msim.restype = C.c_int
        _lib.oracle_xmi_main_msim.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int64, dp, dp, dp,
                                              C.POINTER(C.c_long)]
        _lib.oracle_solid_angle_points.restype = None
        _lib.oracle_solid_angle_points.argtypes = [C.c_void_p, dp, C.c_int, dp, C.c_int64, C.c_int64, C.c_long, dp]
        _lib.oracle_poly_solve_quadratic.restype = C.c_int
        _lib.oracle_poly_solve_quadratic.argtypes = [C.c_double, C.c_double, C.c_double, dp, dp]
        _lib.oracle_words_counted.restype = C.c_longlong
        _lib.oracle_words_counted.argtypes = [C.POINTER(C.c_longlong)]
        _lib.oracle_philox_block.restype = None
        _lib.oracle_philox_block.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        _lib.oracle_solid_angle_points_cl_stream.restype = None
        _lib.oracle_solid_angle_points_cl_stream.argtypes = [C.c_void_p, dp, dp, C.POINTER(C.c_int),
                                                             C.POINTER(C.c_int), C.c_int, C.c_long, dp]
        _lib.oracle_threefry_block.restype = None
        _lib.oracle_threefry_block.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        _lib.oracle_escape_ratios.restype = C.c_int
        _lib.oracle_escape_ratios.argtypes = [C.c_void_p, C.c_long, C.c_double, C.c_double, C.c_long, C.c_long,
                                              C.c_double, C.c_double, C.c_int, dp, dp, dp]
        _lib.oracle_convolute_spectrum.restype = C.c_int
        _lib.oracle_convolute_spectrum.argtypes = [dp, dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                                   C.c_int, C.c_double, C.c_double, C.POINTER(OracleEscape), C.c_int,
                                                   C.c_uint64, dp]
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def escape_ratios(bundle_ptr: int, n_elem: int, n_input: int, e_min: float, e_delta: float, n_photons: int,
                  n_compton: int, c_min: float, c_delta: float, threads: int = 0):
    """Raw sums of the escape-ratio Monte Carlo (oracle_escape_ratios):
    fluo[nE][n_elem][109], comp[nE][nco], interacted[nE]."""
    fluo = np.zeros(n_input * n_elem * 109)
    comp = np.zeros(n_input * n_compton)
    inter = np.zeros(n_input)
    if load().oracle_escape_ratios(C.c_void_p(bundle_ptr), n_input, e_min, e_delta, n_photons, n_compton, c_min,
                                   c_delta, threads, _dp(fluo), _dp(comp), _dp(inter)) != 1:
        raise RuntimeError("oracle escape ratios failed")
    return fluo.reshape(n_input, n_elem, 109), comp.reshape(n_input, n_compton), inter


def msim(bundle_ptr: int, n_interactions: int, nchannels: int, n_mpi_hosts: int = 1, threads: int = 0,
         max_photons_per_item: int = -1) -> dict:
    lib = load()
    ch = np.zeros((n_interactions + 1) * nchannels)
    br = np.zeros(100 * 385 * n_interactions)
    vr = np.zeros(100 * 385 * n_interactions)
    nf = C.c_long(0)
    rv = lib.oracle_xmi_main_msim(C.c_void_p(bundle_ptr), n_mpi_hosts, threads, max_photons_per_item, _dp(ch),
                                  _dp(br), _dp(vr), C.byref(nf))
    if rv != 1:
        raise RuntimeError("oracle transport failed")
    return {"channels": ch.reshape(n_interactions + 1, nchannels), "brute": br.reshape(100, 385, n_interactions),
            "var_red": vr.reshape(100, 385, n_interactions), "not_found": nf.value}


def words_counted() -> int:
    """Algorithmic table words read by the oracle since the previous call."""
    return int(load().oracle_words_counted(None))


def words_counted_split() -> tuple[int, int]:
    """(all words, words of the estimator's element and line loops) since the previous call."""
    est = C.c_longlong(0)
    total = int(load().oracle_words_counted(C.byref(est)))
    return total, int(est.value)


def solid_angle_points(bundle_ptr: int, r_vals: np.ndarray, t_vals: np.ndarray, p0: int, p1: int,
                       hits_per_single: int = 5000) -> np.ndarray:
    lib = load()
    out = np.zeros(p1 - p0)
    r = np.ascontiguousarray(r_vals, dtype=np.float64)
    t = np.ascontiguousarray(t_vals, dtype=np.float64)
    lib.oracle_solid_angle_points(C.c_void_p(bundle_ptr), _dp(r), len(r), _dp(t), p0, p1, hits_per_single, _dp(out))
    return out


def solid_angle_points_cl_stream(bundle_ptr: int, r_vals: np.ndarray, t_vals: np.ndarray, ir, it,
                                 hits_per_single: int = 5000) -> np.ndarray:
    """Grid points (ir[k], it[k]) with the OpenCL kernel's Threefry stream."""
    lib = load()
    r = np.ascontiguousarray(r_vals, dtype=np.float64)
    t = np.ascontiguousarray(t_vals, dtype=np.float64)
    ir = np.ascontiguousarray(ir, dtype=np.int32)
    it = np.ascontiguousarray(it, dtype=np.int32)
    out = np.zeros(len(ir))
    ip = C.POINTER(C.c_int)
    lib.oracle_solid_angle_points_cl_stream(C.c_void_p(bundle_ptr), _dp(r), _dp(t), ir.ctypes.data_as(ip),
                                            it.ctypes.data_as(ip), len(ir), hits_per_single, _dp(out))
    return out


def threefry_block(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 4)(*key)
    o = (C.c_uint32 * 4)()
    lib.oracle_threefry_block(c, k, o)
    return list(o)


REF_CL_LIB = Path(__file__).resolve().parent / "_ref" / "libref_cl.so"


def ref_cl_solid_angle_points(r_vals, t_vals, ir, it, collimator_present: int, detector_radius: float,
                              collimator_radius: float, collimator_height: float, hits_per_single: int = 5000):
    """The reference's own OpenCL solid-angle kernel run on the host
    (oracle/_ref/libref_cl.so, built by oracle/ref_cl/Makefile from the
    reference tree).  FP32 axes and results, as the reference uploads them."""
    lib = C.CDLL(str(REF_CL_LIB))
    f = lib.ref_cl_solid_angle_points
    fp, ip = C.POINTER(C.c_float), C.POINTER(C.c_int)
    f.restype = None
    f.argtypes = [fp, C.c_int, fp, C.c_int, ip, ip, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, fp]
    r = np.ascontiguousarray(r_vals, dtype=np.float32)
    t = np.ascontiguousarray(t_vals, dtype=np.float32)
    ir = np.ascontiguousarray(ir, dtype=np.int32)
    it = np.ascontiguousarray(it, dtype=np.int32)
    out = np.zeros(len(ir), dtype=np.float32)
    f(r.ctypes.data_as(fp), len(r), t.ctypes.data_as(fp), len(t), ir.ctypes.data_as(ip), it.ctypes.data_as(ip),
      len(ir), collimator_present, detector_radius, collimator_radius, collimator_height, hits_per_single,
      out.ctypes.data_as(fp))
    return out


def ref_cl_threefry_block(ctr, key):
    lib = C.CDLL(str(REF_CL_LIB))
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 4)(*key)
    o = (C.c_uint32 * 4)()
    lib.ref_cl_threefry4x32(c, k, o)
    return list(o)


def poly_solve_quadratic(a: float, b: float, c: float):
    lib = load()
    r1, r2 = C.c_double(0.0), C.c_double(0.0)
    n = lib.oracle_poly_solve_quadratic(a, b, c, C.byref(r1), C.byref(r2))
    return n, r1.value, r2.value


def philox_block(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.oracle_philox_block(c, k, o)
    return list(o)


def convolute_spectrum(noconv, det_corr, gain, zero, fano, noise, det_type, live_time, pulse_width,
                       escape: OracleEscape | None = None, use_sum_peaks: int = 0, pile_seed: int = 0):
    lib = load()
    nc = np.ascontiguousarray(noconv, dtype=np.float64)
    dc = np.ascontiguousarray(det_corr, dtype=np.float64)
    out = np.zeros_like(nc)
    rv = lib.oracle_convolute_spectrum(_dp(nc), _dp(dc), len(nc), gain, zero, fano, noise, det_type, live_time,
                                       pulse_width, C.byref(escape) if escape is not None else None, use_sum_peaks,
                                       pile_seed, _dp(out))
    if rv != 1:
        raise RuntimeError("oracle convolution failed")
    return out


def poisson(channels, seed: int):
    """oracle_poisson: Poisson noise on a copy of channels, channel i drawn from
    the Philox stream (seed, i, 0xE0000000)."""
    lib = load()
    f = lib.oracle_poisson
    f.restype, f.argtypes = None, [C.POINTER(C.c_double), C.c_int, C.c_uint64]
    ch = np.array(channels, dtype=np.float64, copy=True)
    f(_dp(ch), len(ch), seed)
    return ch


def sum_peaks(channels, live_time: float, pulse_width: float, gain: float, zero: float, seed: int):
    """oracle_sum_peaks: the pile-up pulse train on a copy of channels."""
    lib = load()
    f = lib.oracle_sum_peaks
    f.restype = C.c_int
    f.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint64]
    ch = np.array(channels, dtype=np.float64, copy=True)
    if f(_dp(ch), len(ch), live_time, pulse_width, gain, zero, seed) != 1:
        raise RuntimeError("oracle pulse train: more than 100 pulses in one group")
    return ch


def compton_qimax(energy: float, binding: float, theta: float) -> float:
    f = load().oracle_compton_qimax
    f.restype, f.argtypes = C.c_double, [C.c_double] * 3
    return f(energy, binding, theta)


def compton_q_from_energy(old_e: float, new_e: float, theta: float) -> float:
    f = load().oracle_compton_q_from_energy
    f.restype, f.argtypes = C.c_double, [C.c_double] * 3
    return f(old_e, new_e, theta)


def compton_energy_from_q(energy: float, q: float, theta: float) -> tuple[float, int]:
    """(scattered energy, error flag): the flag is set where the reference stops."""
    f = load().oracle_compton_energy_from_q
    f.restype, f.argtypes = C.c_double, [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int)]
    err = C.c_int(0)
    return f(energy, q, theta, C.byref(err)), err.value


def compton_shells(bundle_ptr: int, e: int):
    """(shell indices, occupancies, binding energies) of element e's Compton profiles."""
    lib = load()
    sh = (C.c_int * 32)()
    occ, edge = np.zeros(32), np.zeros(32)
    n = lib.oracle_compton_shells(C.c_void_p(bundle_ptr), e, sh, _dp(occ), _dp(edge))
    if n < 0:
        raise RuntimeError("no Compton profile tables in this bundle")
    return np.array(sh[:n]), occ[:n], edge[:n]


def compton_rows(bundle_ptr: int, e: int, k: int, n: int = 10001):
    cdf, qinv = np.zeros(n), np.zeros(n)
    load().oracle_compton_rows(C.c_void_p(bundle_ptr), e, k, _dp(cdf), _dp(qinv))
    return cdf, qinv


def compton_energy_advanced(bundle_ptr: int, e: int, energy: float, theta: float, photon_id: int, stream: int):
    """(scattered energy, shell cumulative values, error flag) of one transport draw."""
    f = load().oracle_compton_energy_advanced
    f.restype = C.c_double
    f.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_uint32, C.POINTER(C.c_double),
                  C.POINTER(C.c_int)]
    cdfs = np.zeros(32)
    err = C.c_int(0)
    E = f(C.c_void_p(bundle_ptr), e, energy, theta, photon_id, stream, _dp(cdfs), C.byref(err))
    return E, cdfs, err.value
