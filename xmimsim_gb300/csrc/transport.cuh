/*
 * Photon transport and the point-detector variance-reduction estimator:
 * the per-photon device functions.  Behaviour follows the reference step for
 * step (src/xmi_main.F90:1188-1685 xmi_simulate_photon and the interaction
 * routines, src/xmi_variance_reduction.F90:29-1101); the structure is the
 * GPU's own:
 *  - the functions here work on one photon (or one estimator event) at a
 *    time; the event-based kernels of wavefront.cuh run them over queues:
 *    a step kernel moves every active photon to its next interaction point
 *    and files it into the Rayleigh, Compton or photo-absorption queue, and
 *    one interaction kernel per queue runs a single code path over its
 *    lanes (escape_kernel in detector.cu still runs whole histories);
 *  - random numbers from Philox streams keyed (photon, phase, draw), so a
 *    photon's sequence does not depend on the launch shape, the queue it
 *    waits in or the kernel that resumes it;
 *  - layer loops fully unrolled over XMI_MAXL with predicates, keeping the
 *    per-layer attenuation state in registers;
 *  - one energy-grid location per energy change, reused by every table;
 *  - the geometric part of the estimator (vr_prologue) runs in the step
 *    kernel and emits one event per interaction; the element and line loops
 *    run later in estimator.cuh over events sorted by (configuration, layer,
 *    order), with FP64 tallies.
 */
#ifndef XMIMSIM_GB300_TRANSPORT_CUH
#define XMIMSIM_GB300_TRANSPORT_CUH

#include "dev_bundle.cuh"

#include <type_traits>

namespace xmi {

enum : unsigned long long { kErrNone = 0, kErrGeometry = 1, kErrTable = 2, kErrCompton = 3,
                            kErrSource = 4, kErrLayer = 5, kErrQueue = 6 };

template <typename R>
struct Photon {
  double c[3];
  R d[3], el[3];
  R theta, phi, E, w, we;
  R mus[XMI_MAXL];
  int layer, elem, n_int, last, inside, hit;
  int h_type, h_elem, h_slot; /* most recent recorded interaction */
  long long id;
};

__device__ __forceinline__ void set_error(const DevTally &t, unsigned long long code) {
  atomicCAS(&t.counters[1], 0ull, code);
}

/* Diagnostic build (-DXMI_CHECKED): every table load and tally store is
 * bounds-checked; the first violation is recorded in xmi_check_record
 * (tag, index, limit, count) and the access is skipped instead of faulting. */
#ifdef XMI_CHECKED
static __device__ unsigned long long xmi_check_record[4];
static __device__ __noinline__ bool xmi_check(long long idx, long long lim, int tag) {
  if (idx >= 0 && idx < lim) return true;
  if (atomicCAS(&xmi_check_record[0], 0ull, (unsigned long long)tag) == 0ull) {
    xmi_check_record[1] = (unsigned long long)idx;
    xmi_check_record[2] = (unsigned long long)lim;
  }
  atomicAdd(&xmi_check_record[3], 1ull);
  return false;
}
template <typename T>
__device__ __forceinline__ T xmi_ldg_checked(const T *p, long long idx, long long lim, int tag) {
  return xmi_check(idx, lim, tag) ? __ldg(p + idx) : (T)0;
}
#define XMI_LDG(p, idx, lim, tag) xmi::xmi_ldg_checked((p), (long long)(idx), (long long)(lim), (tag))
#define XMI_CHK(idx, lim, tag) xmi::xmi_check((long long)(idx), (long long)(lim), (tag))
#else
#define XMI_LDG(p, idx, lim, tag) __ldg((p) + (idx))
#define XMI_CHK(idx, lim, tag) true
#endif

/* ---------------- math helpers ---------------- */
template <typename R> __device__ __forceinline__ R rdot(const R *a, const R *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename R> __device__ __forceinline__ void rnorm(R *a) {
  R n = sqrt(rdot(a, a));
  a[0] /= n; a[1] /= n; a[2] /= n;
}
template <typename R> __device__ __forceinline__ void matvec(const double *m, const R *v, R *r) {
  r[0] = (R)m[0] * v[0] + (R)m[1] * v[1] + (R)m[2] * v[2];
  r[1] = (R)m[3] * v[0] + (R)m[4] * v[1] + (R)m[5] * v[2];
  r[2] = (R)m[6] * v[0] + (R)m[7] * v[1] + (R)m[8] * v[2];
}
template <typename R> __device__ __forceinline__ void matvec_r(const R *m, const R *v, R *r) {
  r[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
  r[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
  r[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}
__device__ __forceinline__ void matvec_d(const double *m, const double *v, double *r) {
  r[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
  r[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
  r[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}

/* distance from p along direction d (unit) to the plane z' = zp of the sample
 * frame (normal n), computed in FP64: xmi_intersection_plane_line +
 * xmi_distance_two_points */
template <typename R>
__device__ __forceinline__ bool plane_step(const double *p, const R *d, const double *n, double zp,
                                           double *ip, double *dist) {
  double dd[3] = {(double)d[0], (double)d[1], (double)d[2]};
  double itn = dd[0] * n[0] + dd[1] * n[1] + dd[2] * n[2];
  if (itn == 0.0) return false;
  double s = ((0.0 - p[0]) * n[0] + (0.0 - p[1]) * n[1] + (zp - p[2]) * n[2]) / itn;
  ip[0] = s * dd[0] + p[0];
  ip[1] = s * dd[1] + p[1];
  ip[2] = s * dd[2] + p[2];
  if (dist) { /* the distance is optional: the first-layer shift does not use it */
    double e0 = p[0] - ip[0], e1 = p[1] - ip[1], e2 = p[2] - ip[2];
    *dist = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
  }
  return true;
}

/* Walk along a fixed direction through the parallel layer planes.  A point x
 * is at height dot(x, n); the boundary plane zp of the sample frame (through
 * (0, 0, zp)) is at height zp * n[2].  One division per direction instead of
 * one per plane: the parametric step to the next plane is its height
 * difference times 1/dot(d, n), and the path length is |step| x |d| (the
 * reference intersects each plane and measures the distance, which is the
 * same quantity). */
struct PlaneWalk {
  double h, inv, dlen;
  float invf, dlenf; /* FP32 transport: the same in FP32 */
};

template <typename R>
__device__ __forceinline__ bool plane_walk_init(const double *p, const R *d, const double *n, PlaneWalk &w,
                                                const R *nr = nullptr) {
  w.h = p[0] * n[0] + p[1] * n[1] + p[2] * n[2];
  if constexpr (sizeof(R) == 4) {
    /* FP32 transport: the direction is FP32, so are 1/cos and |d| (relative
     * error ~1e-7 on the steps); only the heights stay FP64.  This keeps the
     * FP64 divide and square root, slow on this GPU, off the step */
    const float itn = nr ? d[0] * nr[0] + d[1] * nr[1] + d[2] * nr[2]
                         : d[0] * (float)n[0] + d[1] * (float)n[1] + d[2] * (float)n[2];
    if (itn == 0.0f) return false;
    w.invf = 1.0f / itn;
    w.dlenf = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    w.inv = (double)w.invf;
    w.dlen = (double)w.dlenf;
  } else {
    const double dd[3] = {(double)d[0], (double)d[1], (double)d[2]};
    const double itn = dd[0] * n[0] + dd[1] * n[1] + dd[2] * n[2];
    if (itn == 0.0) return false;
    w.inv = 1.0 / itn;
    w.dlen = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
  }
  return true;
}

/* moves point c along the unit sample normal n so that its height c . n
 * becomes h (FP64) */
__device__ __forceinline__ void set_height(double *c, const double *n, double h) {
  const double dh = h - (c[0] * n[0] + c[1] * n[1] + c[2] * n[2]);
  c[0] += dh * n[0];
  c[1] += dh * n[1];
  c[2] += dh * n[2];
}

/* signed parametric step to boundary plane zp; the walk moves onto it */
__device__ __forceinline__ double plane_walk(PlaneWalk &w, double zp, const double *n) {
  const double P = zp * n[2];
  const double s = (P - w.h) * w.inv;
  w.h = P;
  return s;
}

/* Path length from the walk's position through layer j toward its far
 * boundary (up: zend[j], down: zbeg[j]), the walk moving onto it.  FP64 for
 * the first boundary (a difference of heights ~100 cm from the origin), then,
 * in the FP32 transport, the layers' own thicknesses along the normal times
 * 1/cos in FP32: one FP64 subtraction per walk instead of three FP64 ops
 * per crossed boundary. */
template <typename R>
__device__ __forceinline__ double layer_path(const DevBundle<R> &b, PlaneWalk &w, int j, bool up, bool &first) {
  if constexpr (sizeof(R) == 4) {
    float s;
    if (first) {
      const double P = (up ? b.zend[j] : b.zbeg[j]) * b.n_sample[2];
      s = (float)(P - w.h) * w.invf;
      first = false;
    } else {
      s = (float)b.thick_n[j] * w.invf;
    }
    return (double)(fabsf(s) * w.dlenf);
  } else {
    first = false;
    return fabs(plane_walk(w, up ? b.zend[j] : b.zbeg[j], b.n_sample)) * w.dlen;
  }
}

/* uniform draw in the working precision; FP32 uses the rounded FP64 draw so
 * that FP32 and FP64 runs consume identical random sequences */
template <typename R> __device__ __forceinline__ R uni(xmi_rng *g);
template <> __device__ __forceinline__ double uni<double>(xmi_rng *g) { return xmi_rng_uniform(g); }
template <> __device__ __forceinline__ float uni<float>(xmi_rng *g) {
  /* the same two words as the FP64 draw, truncated to 24 bits: within one
   * FP32 ulp of the FP64 run's value, without FP64 arithmetic */
  return (float)(xmi_rng_word(g) >> 8) * 0x1p-24f;
}

/* energy-grid location, same rule as xmi_grid_locate of the bundle, in the
 * working precision (the FP32 build keeps the FP64 pipe free) */
template <typename R>
__device__ __forceinline__ void locate(const DevBundle<R> &b, R E, int &node, R &f) {
  if (E <= __ldg(b.seg_lo)) { node = 0; f = (R)0; return; }
  if (E >= __ldg(b.seg_lo + b.n_seg)) { node = b.n_nodes - 2; f = (R)1; return; }
  /* the segment with seg_lo[lo] <= E < seg_lo[lo + 1] (the bisection's
   * answer): a guess from the search table, then steps until both hold */
  const R lnE = log(E);
  R gb = (lnE - b.seg_lut_ln0) * b.seg_lut_inv;
  gb = gb > (R)0 ? (gb < (R)(XMI_SEG_LUT - 1) ? gb : (R)(XMI_SEG_LUT - 1)) : (R)0;
  int lo = __ldg(b.seg_lut + (int)gb);
#ifndef XMI_CHECKED
  if constexpr (sizeof(R) == 4) {
    /* FP32: the segment's bounds, log base, 1/h, first node and node count
     * in two loads issued together; the steps below only when the table's
     * cell straddles a segment boundary (the same segment either way) */
    float4 r = __ldg(b.seg_rec + lo);
    int2 on = __ldg(b.seg_on + lo);
    if (!(E >= r.x && E < r.y)) {
      while (lo < b.n_seg - 1 && E >= __ldg(b.seg_lo + lo + 1)) lo++;
      while (lo > 0 && E < __ldg(b.seg_lo + lo)) lo--;
      r = __ldg(b.seg_rec + lo);
      on = __ldg(b.seg_on + lo);
    }
    const float t = (lnE - r.z) * r.w;
    int i = (int)t;
    if (i < 0) i = 0;
    if (i > on.y - 2) i = on.y - 2;
    node = on.x + i;
    f = t - (float)i;
    return;
  }
#endif
  while (lo < b.n_seg - 1 && E >= __ldg(b.seg_lo + lo + 1)) lo++;
  while (lo > 0 && E < __ldg(b.seg_lo + lo)) lo--;
  R t = (lnE - __ldg(b.seg_lnlo + lo)) * __ldg(b.seg_invh + lo);
  int i = (int)t;
  int n = __ldg(b.seg_n + lo);
  if (i < 0) i = 0;
  if (i > n - 2) i = n - 2;
  node = b.seg_off[lo] + i;
  f = t - (R)i;
}

template <typename R>
__device__ __forceinline__ R el_val(const DevBundle<R> &b, int e, int col, int node, R f) {
  const long long base = ((long long)e * b.n_nodes + node) * XMI_EL_REC + col;
  const long long lim = (long long)b.n_elem * b.n_nodes * XMI_EL_REC;
  R v0 = XMI_LDG(b.el_tab, base, lim, 1), v1 = XMI_LDG(b.el_tab, base + XMI_EL_REC, lim, 1);
  return v0 + f * (v1 - v0);
}

/* the 9 cascade-corrected shell probabilities of element e at (node, f);
 * FP32 reads each node's 9 values as two 16-byte loads and one word */
template <typename R>
__device__ __forceinline__ void el_xrf(const DevBundle<R> &b, int e, int node, R f, R *P) {
#ifndef XMI_CHECKED
  if constexpr (sizeof(R) == 4 && XMI_REC_XRF % 4 == 0 && XMI_EL_REC % 4 == 0) {
    const float *r0 = b.el_tab + ((long long)e * b.n_nodes + node) * XMI_EL_REC + XMI_REC_XRF;
    const float *r1 = r0 + XMI_EL_REC;
    const float4 a0 = __ldg(reinterpret_cast<const float4 *>(r0)), a1 = __ldg(reinterpret_cast<const float4 *>(r0) + 1);
    const float4 c0 = __ldg(reinterpret_cast<const float4 *>(r1)), c1 = __ldg(reinterpret_cast<const float4 *>(r1) + 1);
    const float a8 = __ldg(r0 + 8), c8 = __ldg(r1 + 8);
    const float v0[9] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w, a8};
    const float v1[9] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w, c8};
#pragma unroll
    for (int s = 0; s < 9; s++) P[s] = v0[s] + f * (v1[s] - v0[s]);
    return;
  }
#endif
#pragma unroll
  for (int s = 0; s < XMI_NSHELL; s++) P[s] = el_val(b, e, XMI_REC_XRF + s, node, f);
}

template <typename R>
__device__ __forceinline__ void mu_calc(const DevBundle<R> &b, R E, R *mus) {
  int node;
  R f;
  locate(b, E, node, f);
  const long long base = (long long)node * XMI_MAXL, lim = (long long)b.n_nodes * XMI_MAXL;
#ifndef XMI_CHECKED
  if constexpr (sizeof(R) == 4 && XMI_MAXL == 8) {
    /* the two 32-byte node rows as four 16-byte loads */
    const float4 *p = reinterpret_cast<const float4 *>(b.mu_tab + base);
    const float4 a0 = __ldg(p), a1 = __ldg(p + 1), c0 = __ldg(p + 2), c1 = __ldg(p + 3);
    const float v0[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
    const float v1[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
    for (int j = 0; j < 8; j++) mus[j] = v0[j] + f * (v1[j] - v0[j]);
    return;
  }
#endif
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++) {
    R v0 = XMI_LDG(b.mu_tab, base + j, lim, 2), v1 = XMI_LDG(b.mu_tab, base + XMI_MAXL + j, lim, 2);
    mus[j] = v0 + f * (v1 - v0);
  }
}

/* findpos (src/xmi_aux_f.F90:1305) on a uniform axis: same result as the
 * linear scan, found from an arithmetic guess and a +-1 correction */
template <typename R>
__device__ __forceinline__ int findpos_u(const R *a, int n, R x, R a0, R inv_dx) {
  /* NaN never compares <= an axis value: not found (the linear scan's answer).
   * The guess is clamped in floating point before the integer conversion,
   * since an FP64 NaN converts to INT_MIN. */
  if (!(x == x)) return -1;
  if (fabs(x - XMI_LDG(a, 0, n, 3)) < (R)1e-10) return 0;
  R gr = ceil((x - a0) * inv_dx);
  int i = !(gr >= (R)1) ? 1 : (!(gr <= (R)(n - 1)) ? n - 1 : (int)gr);
  while (i > 1 && x <= XMI_LDG(a, i - 1, n, 3)) i--;
  while (i < n && x > XMI_LDG(a, i, n, 3)) i++;
  return i >= n ? -1 : i - 1;
}

/* bilinear_interpolation (src/xmi_aux_f.F90:1337) of a2[i2*n1+i1] */
template <typename R>
__device__ __forceinline__ R bilinear(const R *a2, const R *a, int n1, R a0, R ainv, const R *bb, int n2, R b0,
                                      R binv, R x1, R x2, bool &ok) {
  int p1 = findpos_u(a, n1, x1, a0, ainv), p2 = findpos_u(bb, n2, x2, b0, binv);
  if (p1 < 0 || p2 < 0) { ok = false; return (R)0; }
  R a_0 = XMI_LDG(a, p1, n1, 4), a_1 = XMI_LDG(a, p1 + 1, n1, 4), b_0 = XMI_LDG(bb, p2, n2, 4),
    b_1 = XMI_LDG(bb, p2 + 1, n2, 4);
  R denom = (a_1 - a_0) * (b_1 - b_0);
  R c1 = (a_1 - x1) * (b_1 - x2) / denom;
  R c2 = (x1 - a_0) * (b_1 - x2) / denom;
  R c3 = (a_1 - x1) * (x2 - b_0) / denom;
  R c4 = (x1 - a_0) * (x2 - b_0) / denom;
  const long long o = (long long)p2 * n1 + p1, lim = (long long)n1 * n2;
  return c1 * XMI_LDG(a2, o, lim, 5) + c2 * XMI_LDG(a2, o + 1, lim, 5) + c3 * XMI_LDG(a2, o + n1, lim, 5) +
         c4 * XMI_LDG(a2, o + n1 + 1, lim, 5);
}

template <typename R>
__device__ __forceinline__ R qtab(const R *t, R q) {
  R x = q * (R)((XMI_NQ - 1) / XMI_QMAX);
  int i = (int)x;
  if (i < 0) i = 0;
  if (i > XMI_NQ - 2) i = XMI_NQ - 2;
  R f = x - (R)i;
  R v0 = XMI_LDG(t, i, XMI_NQ, 6), v1 = XMI_LDG(t, i + 1, XMI_NQ, 6);
  return v0 + f * (v1 - v0);
}

/* visits the layers in the direction of travel with compile-time indices
 * (both orders fully unrolled) so per-layer arrays stay in registers */
template <typename F>
__device__ __forceinline__ void layers_in_direction(bool up, F &&f) {
  if (up) {
#pragma unroll
    for (int j = 0; j < XMI_MAXL; j++) f(j);
  } else {
#pragma unroll
    for (int j = XMI_MAXL - 1; j >= 0; j--) f(j);
  }
}

template <typename R>
__device__ __forceinline__ R select_layer(const R *v, int layer) {
  R out = (R)0;
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++)
    if (j == layer) out = v[j];
  return out;
}

/* ---------------- tallies ---------------- */
__device__ __forceinline__ double warp_sum(unsigned mask, double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off);
  return v;
}

/* atomicAdd with warp pre-reduction when every active lane targets the same
 * address (the common case in the estimator's element and line loops) */
__device__ __forceinline__ void tally_add(double *addr, double v) {
  unsigned mask = __activemask();
  int pred;
  __match_all_sync(mask, (unsigned long long)addr, &pred);
  if (pred && mask == 0xffffffffu) {
    double s = warp_sum(mask, v);
    if ((threadIdx.x & 31) == 0) atomicAdd(addr, s);
  } else {
    atomicAdd(addr, v);
  }
}

/* channel of energy E: INT((E - zero) / gain), src/xmi_main.F90 (tallies);
 * evaluated in the working precision */
template <typename R>
__device__ __forceinline__ int channel_of(const DevBundle<R> &b, R E) {
  /* FP32: a multiply by 1/gain (a channel edge may move by an ulp) */
  if constexpr (sizeof(R) == 4) return (int)((E - b.zero_r) * b.inv_gain_r);
  else return (int)((E - (R)b.zero) / (R)b.gain);
}

template <typename R>
__device__ __forceinline__ void tally_channel(const DevBundle<R> &b, const DevTally &t, int n, R E, double w) {
  int ch = -1;
  if (E >= (R)kEnergyThreshold) ch = channel_of(b, E);
  if (ch >= 0 && ch <= b.nch - 1 && XMI_CHK((long long)n * b.nch + ch, (long long)(b.N + 1) * b.nch, 30))
    tally_add(&t.chan[(size_t)n * b.nch + ch], w);
}

/* ---------------- solid angle ---------------- */
/* distance and angle of a point to the collimator's opening: the reference
 * computes r = sqrt(r1^2 - 2 r1 sin(theta1) h + h^2) and theta =
 * acos(r1 cos(theta1) / r).  In FP32 that difference cancels when the point
 * lies near the height of the opening, and rounding can push the cosine
 * above 1 (a NaN solid angle, seen on the collimated workload at 1e8
 * photons); the FP32 engine uses the exact rewriting r^2 = py^2 + (pz - h)^2
 * with py = r1 cos(theta1), pz = r1 sin(theta1), and theta = atan2(|pz - h|,
 * py), which neither cancels nor leaves the cosine's range.  FP64 keeps the
 * reference's arithmetic. */
template <typename R>
__device__ __forceinline__ void sa_opening(R r1, R theta1, R collh, R &r, R &theta) {
  if constexpr (sizeof(R) == 4) {
    const R py = r1 * cos(theta1), dz = fabs(r1 * sin(theta1) - collh);
    r = sqrt(py * py + dz * dz);
    theta = atan2(dz, py);
  } else {
    r = sqrt(r1 * r1 - (R)2.0 * r1 * sin(theta1) * collh + collh * collh);
    theta = acos(r1 * cos(theta1) / r);
  }
}

/* xmi_single_solid_angle_calculation (src/xmi_solid_angle_f.F90:432-710) */
template <typename R>
__device__ R single_solid_angle(const DevBundle<R> &b, R r1, R theta1, xmi_rng *g, int hits_per_single) {
  R r, theta, fcbr;
  bool outside;
  const R detr = (R)b.det_radius, collr = (R)b.coll_radius, collh = (R)b.coll_height;
  if (!b.coll_present) {
    r = r1; theta = theta1; fcbr = detr; outside = false;
  } else if (fabs(collr - detr) < (R)0.000001) {
    if (r1 * cos(theta1) <= detr) {
      r = r1; theta = theta1; fcbr = detr;
    } else {
      sa_opening<R>(r1, theta1, collh, r, theta);
      fcbr = collr;
    }
    outside = r1 * sin(theta1) > collh;
  } else {
    if (r1 * cos(theta1) <= detr && r1 * sin(theta1) <= collh * (r1 * cos(theta1) - detr) / (collr - detr)) {
      r = r1; theta = theta1; fcbr = detr;
    } else if (r1 * sin(theta1) <= collh) {
      return (R)0;
    } else {
      sa_opening<R>(r1, theta1, collh, r, theta);
      fcbr = collr;
    }
    outside = r1 * sin(theta1) > collh;
  }
  R beta = atan(fcbr / r);
  R alpha1 = atan(fcbr * sin(theta) / (r - fcbr * cos(theta)));
  if (alpha1 <= (R)0) alpha1 = alpha1 + (R)kPi;
  R fca = beta > alpha1 ? beta : alpha1;
  R cfca = cos(fca);
  R fcsa = (R)(2 * kPi) * ((R)1 - cfca);
  R st = sin(theta), ct = cos(theta);
  R py = r1 * cos(theta1), pz = r1 * sin(theta1);
  int hits = 0;
  for (int i = 0; i < hits_per_single; i++) {
    R th = acos((R)1 - uni<R>(g) * ((R)1 - cfca));
    R ph = uni<R>(g) * (R)2 * (R)kPi;
    R sth = sin(th);
    R dcx = sth * cos(ph), dcy = sth * sin(ph), dcz = cos(th);
    /* rotation rows (1,0,0), (0,-sin,-cos), (0,cos,-sin) */
    R dx = dcx, dy = -st * dcy - ct * dcz, dz = ct * dcy - st * dcz;
    if (dz >= (R)0) continue;
    if (outside) {
      R s = (collh - pz) / dz;
      R ix = s * dx, iy = s * dy + py;
      if (sqrt(ix * ix + iy * iy) > collr) continue;
    }
    R s = (-pz) / dz;
    R ix = s * dx, iy = s * dy + py, iz = s * dz + pz;
    if (sqrt(ix * ix + iy * iy + iz * iz) <= detr) hits++;
  }
  return fcsa * (R)hits / (R)hits_per_single;
}

/* a cosine computed from rounded unit vectors, kept in [-1, 1]: on the
 * detector axis the dot product can round one ulp past 1, and acos would
 * return NaN (the grid lookup turned that NaN into the axis end; the
 * surrogate path would have served it a zero solid angle) */
template <typename R>
__device__ __forceinline__ R cos_clamp(R c) {
  return c > (R)1 ? (R)1 : (c < (R)-1 ? (R)-1 : c);
}

/* (r, theta) of a point in the solid-angle grid's frame: distance to the
 * detector centre and the complement of the angle to the detector normal */
template <typename R>
__device__ __forceinline__ void sa_coords(const DevBundle<R> &b, const double *coords, R &r, R &theta) {
  double dv[3] = {coords[0] - b.p_det[0], coords[1] - b.p_det[1], coords[2] - b.p_det[2]};
  R dn[3];
  double rr;
  if constexpr (sizeof(R) == 4) {
    /* the offset from the detector is FP64 (a difference of positions), its
     * length and direction FP32 */
    const float f[3] = {(float)dv[0], (float)dv[1], (float)dv[2]};
    const float rf = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]), inv = 1.0f / rf;
    rr = rf;
    dn[0] = f[0] * inv, dn[1] = f[1] * inv, dn[2] = f[2] * inv;
  } else {
    rr = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    const double inv = 1.0 / rr;
    dn[0] = (R)(dv[0] * inv), dn[1] = (R)(dv[1] * inv), dn[2] = (R)(dv[2] * inv);
  }
  const R *nd = b.n_det_r;
  R tt = acos(cos_clamp(rdot(dn, nd)));
  r = (R)rr;
  if (tt > (R)(kPi / 2.0)) tt = (R)kPi - tt;
  theta = (R)(kPi / 2.0) - tt;
}

/* xmi_get_solid_angle (src/xmi_solid_angle_f.F90:712-801) */
template <typename R>
__device__ R get_solid_angle(const DevBundle<R> &b, const double *coords, const Photon<R> &p, const DevTally &t,
                             bool &ok, bool *deferred = nullptr, R *def_r = nullptr, R *def_t = nullptr) {
  double dv[3] = {coords[0] - b.p_det[0], coords[1] - b.p_det[1], coords[2] - b.p_det[2]};
  R dn[3];
  double rr;
  if constexpr (sizeof(R) == 4) {
    const float f[3] = {(float)dv[0], (float)dv[1], (float)dv[2]};
    const float rf = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]), inv = 1.0f / rf;
    rr = rf;
    dn[0] = f[0] * inv, dn[1] = f[1] * inv, dn[2] = f[2] * inv;
  } else {
    rr = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    const double inv = 1.0 / rr;
    dn[0] = (R)(dv[0] * inv), dn[1] = (R)(dv[1] * inv), dn[2] = (R)(dv[2] * inv);
  }
  const R *nd = b.n_det_r;
  R tt = acos(cos_clamp(rdot(dn, nd)));
  R r = (R)rr;
  if (tt > (R)(kPi / 2.0)) tt = (R)kPi - tt;
  R theta = (R)(kPi / 2.0) - tt;
  if (theta < (R)b.sa_t[0]) return (R)0;
  /* theta <= pi/2 by construction; in FP32, pi/2 itself rounds above the
   * axis end (the FP64 pi/2), which would send every point on the detector
   * axis to the Monte Carlo fallback */
  const double th = fmin((double)theta, b.sa_t[b.sa_nt - 1]);
  int p1 = findpos_u<double>(b.sa_r, b.sa_nr, (double)r, b.sa_r0, b.sa_rinv);
  int p2 = findpos_u<double>(b.sa_t, b.sa_nt, th, b.sa_t0, b.sa_tinv);
  if (p1 == -1 || p2 == -1) {
    atomicAdd(&t.counters[0], 1ull);
    if (deferred) {
      /* the caller leaves the integral to a warp-parallel pass over the
       * queued events (the same draws: sample i is Philox block i of the
       * stream below) */
      *deferred = true;
      *def_r = r;
      *def_t = theta;
      return (R)1;
    }
    xmi_rng g;
    xmi_rng_init(&g, b.seed, (uint64_t)p.id, 0x80000000u | (uint32_t)p.n_int);
    return single_solid_angle(b, r, theta, &g, b.sa_hits);
  }
  /* bilinear on the grid; axes are FP64, values in R */
  double a0 = b.sa_r[p1], a1 = b.sa_r[p1 + 1], b0 = b.sa_t[p2], b1 = b.sa_t[p2 + 1];
  double x1 = (double)r, x2 = th;
  R denom = (R)((a1 - a0) * (b1 - b0));
  R c1 = (R)((a1 - x1) * (b1 - x2)) / denom;
  R c2 = (R)((x1 - a0) * (b1 - x2)) / denom;
  R c3 = (R)((a1 - x1) * (x2 - b0)) / denom;
  R c4 = (R)((x1 - a0) * (x2 - b0)) / denom;
  const long long o = (long long)p2 * b.sa_nr + p1, lim = (long long)b.sa_nr * b.sa_nt;
  (void)ok;
  return c1 * XMI_LDG(b.sa_grid, o, lim, 7) + c2 * XMI_LDG(b.sa_grid, o + 1, lim, 7) +
         c3 * XMI_LDG(b.sa_grid, o + b.sa_nr, lim, 7) + c4 * XMI_LDG(b.sa_grid, o + b.sa_nr + 1, lim, 7);
}

/* ---------------- photon kinematics ---------------- */
/* xmi_update_photon_dirv (src/xmi_main.F90:5071-5148) */
template <typename R>
__device__ __forceinline__ void update_dirv(Photon<R> &p, R theta_i, R phi_i) {
  R phn;
  if (phi_i > (R)(2.0 * kPi)) phn = phi_i - (R)(2.0 * kPi);
  else if (phi_i < (R)0) phn = phi_i + (R)(2.0 * kPi);
  else phn = phi_i;
  R cphi = cos(p.phi), sphi = sin(p.phi), cth = cos(p.theta), sth = sin(p.theta);
  R ts = sin(theta_i);
  R dx = ts * cos(phn), dy = ts * sin(phn), dz = cos(theta_i);
  p.d[0] = cth * cphi * dx - sphi * dy + sth * cphi * dz;
  p.d[1] = cth * sphi * dx + cphi * dy + sth * sphi * dz;
  p.d[2] = -sth * dx + cth * dz;
  rnorm(p.d);
  p.theta = acos(p.d[2]);
  p.phi = atan2(p.d[1], p.d[0]);
  if (p.phi > (R)(2.0 * kPi)) p.phi = p.phi - (R)(2.0 * kPi);
  else if (p.phi < (R)0) p.phi = p.phi + (R)(2.0 * kPi);
}

/* xmi_update_photon_elecv (src/xmi_main.F90:5150-5182) */
template <typename R>
__device__ __forceinline__ void update_elecv(Photon<R> &p) {
  R cosalfa = rdot(p.d, p.el);
  R c_alfa = acos(cosalfa);
  R sinalfa = sin(c_alfa);
  if (!(fabs(sinalfa) > (R)0)) {
    /* direction parallel to the E-vector after rounding (reachable in FP32 only):
     * any unit vector perpendicular to the direction is a valid E-vector, the
     * reference formula would produce inf/NaN here */
    R ax[3] = {(R)0, (R)0, (R)0};
    int k = fabs(p.d[0]) < fabs(p.d[1]) ? (fabs(p.d[0]) < fabs(p.d[2]) ? 0 : 2) : (fabs(p.d[1]) < fabs(p.d[2]) ? 1 : 2);
    ax[k] = (R)1;
    p.el[0] = p.d[1] * ax[2] - p.d[2] * ax[1];
    p.el[1] = p.d[2] * ax[0] - p.d[0] * ax[2];
    p.el[2] = p.d[0] * ax[1] - p.d[1] * ax[0];
    rnorm(p.el);
    return;
  }
  R c_ae = (R)1 / sinalfa, c_be = -c_ae * cosalfa;
#pragma unroll
  for (int k = 0; k < 3; k++) p.el[k] = c_ae * p.el[k] + c_be * p.d[k];
  rnorm(p.el);
}

template <typename R>
__device__ __forceinline__ R polarisation_phi0(const Photon<R> &p) {
  R cphi = cos(p.phi), sphi = sin(p.phi), cth = cos(p.theta), sth = sin(p.theta);
  R cosphi0 = p.el[0] * cphi * cth + p.el[1] * cth * sphi - p.el[2] * sth;
  R sinphi0 = p.el[0] * sphi - p.el[1] * cphi;
  if (fabs(cosphi0) > (R)1) cosphi0 = cosphi0 > (R)0 ? (R)1 : (R)-1;
  R phi0 = acos(cosphi0);
  if (sinphi0 > (R)0) phi0 = -phi0;
  return phi0;
}

/* Doppler-broadened Compton energy: src/xmi_main.F90:4985-5067 (transport)
 * and src/xmi_variance_reduction.F90:1010-1101 (estimator) */
template <typename R>
__device__ __forceinline__ R compton_energy(const DevBundle<R> &b, int e, R E, R theta_i, xmi_rng *g, bool varred,
                                           bool &ok) {
  const R c = (R)(double)1.2399e-6f, c0 = (R)(double)4.85e-12f, c1 = (R)(double)1.456e-2f;
  const R *rn = b.dop_r, *icdf = b.dop_icdf[e];
  const R dr = __ldg(rn + 1) - __ldg(rn);
  R energy = E * (R)1000, c_lamb0 = c / energy, sth2 = sin(theta_i / (R)2);
  int it = 0;
  for (int tries = 0; tries < 100000; tries++) {
    R r = uni<R>(g);
    int pos = (int)(r / dr);
    if (varred && pos == XMI_DOPPLER_N - 2) continue;
    if (pos > XMI_DOPPLER_N - 2) pos = XMI_DOPPLER_N - 2;
    R r0 = XMI_LDG(rn, pos, XMI_DOPPLER_N, 8), r1 = XMI_LDG(rn, pos + 1, XMI_DOPPLER_N, 8);
    R q0 = XMI_LDG(icdf, pos, XMI_DOPPLER_N, 8), q1 = XMI_LDG(icdf, pos + 1, XMI_DOPPLER_N, 8);
    R pz = q0 + ((q1 - q0) * (r - r0) / (r1 - r0));
    if (uni<R>(g) < (R)0.5) pz = -pz;
    R dlamb = c0 * sth2 * sth2 - c1 * c_lamb0 * sth2 * pz;
    R c_lamb = c_lamb0 + dlamb;
    energy = c / c_lamb / (R)1000;
    /* the reference accepts when energy <= E; dlamb >= 0 is the same test in
     * exact arithmetic, and unlike it cannot be defeated by rounding (in FP32
     * c / (c / E) exceeds E for about half of all E, which near theta = 0
     * would reject every draw) */
    if (dlamb >= (R)0) return energy;
    if (varred) {
      if (it == 100) break;
      it++;
    }
  }
  ok = false;
  return (R)0;
}

/* The estimator's Doppler Compton energy (compton_energy with varred) with
 * the per-event factors hoisted out of the element loop: dlamb = k0 - k1 pz.
 * FP64 keeps the table interpolation of the transport; FP32 interpolates the
 * uniform Doppler axis by index arithmetic (no division, two loads fewer). */
template <typename R>
struct ComptonEvent {
  R c_lamb0, k0, k1;
};

template <typename R>
__device__ __forceinline__ ComptonEvent<R> compton_event(R E, R theta_i) {
  const R c = (R)(double)1.2399e-6f, c0 = (R)(double)4.85e-12f, c1 = (R)(double)1.456e-2f;
  const R energy = E * (R)1000, c_lamb0 = c / energy, sth2 = sin(theta_i / (R)2);
  return {c_lamb0, c0 * sth2 * sth2, c1 * c_lamb0 * sth2};
}

template <typename R>
__device__ __forceinline__ R compton_energy_est(const DevBundle<R> &b, int e, const ComptonEvent<R> &ce, xmi_rng *g,
                                               bool &ok) {
  const R c = (R)(double)1.2399e-6f;
  const R *rn = b.dop_r, *icdf = b.dop_icdf[e];
  const R dr = __ldg(rn + 1) - __ldg(rn);
  const R inv_dr = (R)(XMI_DOPPLER_N - 1);
  int it = 0;
  for (int tries = 0; tries < 100000; tries++) {
    const R r = uni<R>(g);
    R pz;
    if constexpr (sizeof(R) == 4) {
      const R tpos = r * inv_dr;
      int pos = (int)tpos;
      if (pos == XMI_DOPPLER_N - 2) continue;
      if (pos > XMI_DOPPLER_N - 2) pos = XMI_DOPPLER_N - 2;
      const R q0 = XMI_LDG(icdf, pos, XMI_DOPPLER_N, 8), q1 = XMI_LDG(icdf, pos + 1, XMI_DOPPLER_N, 8);
      pz = q0 + (q1 - q0) * (tpos - (R)pos);
    } else {
      int pos = (int)(r / dr);
      if (pos == XMI_DOPPLER_N - 2) continue;
      if (pos > XMI_DOPPLER_N - 2) pos = XMI_DOPPLER_N - 2;
      const R r0 = XMI_LDG(rn, pos, XMI_DOPPLER_N, 8), r1 = XMI_LDG(rn, pos + 1, XMI_DOPPLER_N, 8);
      const R q0 = XMI_LDG(icdf, pos, XMI_DOPPLER_N, 8), q1 = XMI_LDG(icdf, pos + 1, XMI_DOPPLER_N, 8);
      pz = q0 + ((q1 - q0) * (r - r0) / (r1 - r0));
    }
    if (uni<R>(g) < (R)0.5) pz = -pz;
    const R dlamb = ce.k0 - ce.k1 * pz;
    if (dlamb >= (R)0) {
      if constexpr (sizeof(R) == 4) return (c / (R)1000) / (ce.c_lamb0 + dlamb); /* one division */
      else return c / (ce.c_lamb0 + dlamb) / (R)1000;
    }
    if (it == 100) break;
    it++;
  }
  ok = false;
  return (R)0;
}

/* ---------------- advanced Compton: per-shell impulse approximation ----------------
 * src/xmi_main.F90:4785-4983 (transport), src/xmi_variance_reduction.F90:752-947
 * (estimator), src/xmi_aux_f.F90:1951-2074 (momentum kinematics).  The FP64
 * engine follows the reference's arithmetic (the oracle's parity).  The FP32
 * engine runs the kinematics in FP32 with the same quadratic solved in a form
 * without cancellation: its discriminant is 4 a^2 Q^2 (K^2 ((d - c)^2 +
 * sin^2 theta) - Q^2 sin^2 theta), the larger root comes directly and the
 * smaller from the product of the roots, and since Q(E) grows with E the root
 * with the sign of Q is the larger one for Q > 0.  FP64 divides and square
 * roots are slow on this GPU; the FP32 form keeps them off the per-shell loop.
 * MEC2 here is xraylib's constant; 1E-8, 1E-4 and 1E-10 are the reference's
 * default-real literals. */
constexpr double kXrlMec2 = 510.998928;

template <typename R>
using cp_real = typename std::conditional<sizeof(R) == 4, float, double>::type;

/* xmi_get_qimax (c = cos theta, h2 = sin^2(theta / 2)).  FP64 follows the
 * reference's arithmetic; FP32 writes 1 - c as 2 h2 and the denominator
 * (E - I)^2 + E^2 - 2 (E - I) E c as I^2 + 4 (E - I) E h2, which are exact
 * rewritings without the cancellation both forms of the reference suffer at
 * small theta (1% error at theta = 5e-3 in FP32). */
template <typename T>
__device__ __forceinline__ T cp_qimax(T energy, T Ii, T c, T h2) {
  if (Ii != (T)0 && energy < Ii) return (T)0;
  const T emi = energy - Ii;
  if constexpr (sizeof(T) == 4) {
    const T q = (T)137 * ((T)2 * emi * energy * h2 / (T)kXrlMec2 - Ii);
    return q / sqrt(Ii * Ii + (T)4 * emi * energy * h2);
  } else {
    const T q = (T)137 * (emi * energy * ((T)1 - c) / (T)kXrlMec2 - Ii);
    return q / sqrt(emi * emi + energy * energy - (T)2 * emi * energy * c);
  }
}

/* xmi_get_q_from_energy */
__device__ __forceinline__ double cp_q_from_energy(double old_e, double new_e, double c) {
  const double q = 137.0 * (new_e - old_e + (1.0 - c) * old_e * new_e / kXrlMec2);
  return q / sqrt(new_e * new_e + old_e * old_e - 2.0 * old_e * new_e * c);
}

/* xmi_get_energy_from_q with xmi_poly_solve_quadratic; bad = true where the
 * reference stops the program (neither root has the sign of Q) */
static __device__ __noinline__ double cp_energy_from_q(double a, double Q, double c, double /*sin theta*/,
                                                       bool &bad) {
  const double b = kXrlMec2, k2 = 137.0 * 137.0;
  if (fabs(c - 1.0) < (double)1e-8f) return 0.0;
  if (fabs(Q) < (double)1e-4f) return a / (1.0 + a * (1.0 - c) / b);
  const double d = 1.0 + a / b - a * c / b;
  const double aq = k2 * (d * d) - Q * Q;
  const double bq = -(2.0 * k2 * a * d) + 2.0 * a * c * (Q * Q);
  const double cq = k2 * (a * a) - (a * a) * (Q * Q);
  double e1, e2;
  if (aq == 0.0) {
    if (bq == 0.0) return 0.0;
    e1 = e2 = -1.0 * cq / bq;
  } else {
    const double delta = bq * bq - 4.0 * aq * cq;
    if (delta < 0.0) return 0.0;
    if (delta == 0.0) {
      e1 = e2 = -bq / 2.0 / aq;
    } else {
      const double sd = sqrt(delta), r1 = (-bq + sd) / 2.0 / aq, r2 = (-bq - sd) / 2.0 / aq;
      e1 = fmin(r1, r2);
      e2 = fmax(r1, r2);
    }
  }
  const double q1 = cp_q_from_energy(a, e1, c), q2 = cp_q_from_energy(a, e2, c);
  if (Q * q1 > 0.0) return e1;
  if (Q * q2 > 0.0) return e2;
  if (fabs(e1 - e2) < (double)1e-10f || fabs(q1 - q2) < (double)1e-10f) return e1;
  bad = true;
  return 0.0;
}

/* the same energy in FP32, the quadratic solved without cancellation (see above) */
__device__ __forceinline__ float cp_energy_from_q(float a, float Q, float c, float s, bool & /*bad*/) {
  const float b = (float)kXrlMec2, k2 = 137.0f * 137.0f;
  if (fabsf(c - 1.0f) < 1e-8f) return 0.0f;
  if (fabsf(Q) < 1e-4f) return a / (1.0f + a * (1.0f - c) / b);
  const float d = 1.0f + a * (1.0f - c) / b;
  const float A = k2 * d * d - Q * Q;                  /* > 0: d >= 1, |Q| <= 100 */
  const float dc = d - c, s2 = s * s;
  const float root = fabsf(Q) * sqrtf(fmaxf(k2 * (dc * dc + s2) - Q * Q * s2, 0.0f));
  const float B = k2 * d - c * Q * Q;                  /* > 0 for |Q| <= 100 */
  const float e_big = a * (B + root) / A;
  return Q > 0.0f ? e_big : a * a * (k2 - Q * Q) / (A * e_big);
}

/* the shell's cumulative profile up to qimax (uniform Q axis, 100 / (N-1)) */
template <typename T, typename R>
__device__ __forceinline__ T cp_shell_cdf(const R *row, T qimax) {
  const T dq = (T)(100.0 * 1.0 / (XMI_CP_N - 1.0) - 100.0 * 0.0 / (XMI_CP_N - 1.0));
  if (qimax != qimax) qimax = (T)0; /* 0/0 at theta = 0 with a zero binding energy: undefined in the reference */
  if (qimax < (T)-100) return (T)0;
  if (qimax > (T)100) return (T)1;
  const T x = qimax < (T)0 ? -qimax : qimax;
  int pos = (int)(x / dq);
  if (pos > XMI_CP_N - 2) pos = XMI_CP_N - 2; /* x = 100 exactly: the last interval */
  const T x0 = (T)100 * (T)pos / (T)(XMI_CP_N - 1.0), x1 = (T)100 * (T)(pos + 1) / (T)(XMI_CP_N - 1.0);
  const T y0 = (T)XMI_LDG(row, pos, XMI_CP_N, 50), y1 = (T)XMI_LDG(row, pos + 1, XMI_CP_N, 50);
  const T v = y0 + ((y1 - y0) * (x - x0) / (x1 - x0));
  return qimax < (T)0 ? (T)1 - ((T)0.5 + v) : (T)0.5 + v;
}

/* the shell's Q at cumulative value cdf (uniform CDF axis, 0.5 / (N-1)) */
template <typename T, typename R>
__device__ __forceinline__ T cp_shell_q(const R *row, T cdf) {
  const T dc = (T)(0.5 * 1.0 / (XMI_CP_N - 1.0) - 0.5 * 0.0 / (XMI_CP_N - 1.0));
  const bool neg = cdf < (T)0.5;
  const T cp = neg ? (T)0.5 - cdf : cdf - (T)0.5;
  int pos = (int)(cp / dc);
  /* the reference stops the program at pos = N - 1 (cdf exactly 0 or 1) */
  if (pos > XMI_CP_N - 2) pos = XMI_CP_N - 2;
  const T c0 = (T)0.5 * (T)pos / (T)(XMI_CP_N - 1.0), c1 = (T)0.5 * (T)(pos + 1) / (T)(XMI_CP_N - 1.0);
  const T y0 = (T)XMI_LDG(row, pos, XMI_CP_N, 51), y1 = (T)XMI_LDG(row, pos + 1, XMI_CP_N, 51);
  const T q = y0 + ((y1 - y0) * (cp - c0) / (c1 - c0));
  return neg ? -q : q;
}

/* every shell's cumulative profile at (energy, c = cos theta) and their
 * occupancy-weighted sum */
template <typename T, typename R>
__device__ __forceinline__ T cp_shell_cdfs(const DevBundle<R> &b, int e, T energy, T c, T h2, T *cdfs) {
  const int ns = b.cp_nshell[e];
  for (int k = 0; k < ns; k++)
    cdfs[k] = cp_shell_cdf<T>(b.cp_cdf[e] + (size_t)k * XMI_CP_N,
                              cp_qimax<T>(energy, (T)b.cp_edge[e * XMI_CP_SH + k], c, h2));
  T sum = (T)0;
  for (int k = 0; k < ns; k++) sum = sum + (T)b.cp_occ[e * XMI_CP_SH + k] * cdfs[k];
  return sum;
}

/* xmi_update_photon_energy_compton: the scattered energy, 0 when no shell can
 * scatter (the photon is then absorbed) */
template <typename R>
__device__ __noinline__ double compton_energy_advanced(const DevBundle<R> &b, int e, double energy_in, double theta_i,
                                                       xmi_rng *g, bool &bad) {
  using T = cp_real<R>;
  T cdfs[XMI_CP_SH];
  const T energy = (T)energy_in, th = (T)theta_i, c = cos(th), sn = sin(th), sh = sin(th * (T)0.5);
  const T sum = cp_shell_cdfs<T>(b, e, energy, c, sh * sh, cdfs);
  if (sum == (T)0) return 0.0;
  const int ns = b.cp_nshell[e];
  const T r = (T)uni<R>(g);
  T tsum = (T)0;
  int sel = -1;
  for (int k = 0; k < ns; k++) {
    const T w = (T)b.cp_occ[e * XMI_CP_SH + k] * cdfs[k] / sum;
    if (w > (T)0) sel = k; /* rounding can leave the running sum below r: the last shell with weight */
    tsum = tsum + w;
    if (r <= tsum) {
      sel = k;
      break;
    }
  }
  if (sel < 0) { /* not reached with finite tables */
    bad = true;
    return 0.0;
  }
  const T q = cp_shell_q<T>(b.cp_qinv[e] + (size_t)sel * XMI_CP_N, (T)uni<R>(g) * cdfs[sel]);
  return (double)cp_energy_from_q(energy, q, c, sn, bad);
}

/* ---------------- variance reduction: event prologue ---------------- */
/* The point-detector estimator of one interaction
 * (src/xmi_variance_reduction.F90:29-726) is split in two.  The transport
 * kernel evaluates the part that depends on the photon's geometry -- a point
 * on the detector, the scattering angles toward it, the path through the
 * layers, the solid angle -- and stores it as one VrEvent; the estimator
 * kernel later evaluates every element and line of the layer for it.  The
 * estimator's random draws come from streams of their own,
 * (photon, 0x40000000 | n << 8 | 0xFF) for the detector point and
 * (photon, 0x40000000 | n << 8 | i) for the Compton energy of the i-th
 * element of the layer, so neither part depends on the other's draws. */
template <typename R>
struct __align__(16) VrEvent {
  R E, w, mu_here;
  R pR, pC;          /* omega x Thomson factor, omega x Klein-Nishina factor */
  R q, theta;        /* momentum transfer, scattering angle toward the detector point */
  R pdir_fluo;       /* omega / 4 pi */
  R pesc_rayl;       /* escape probability at the photon energy */
  R f;               /* energy-grid fraction of E */
  R sa_r, sa_t;      /* the point's (r, theta) of the solid-angle grid (the surrogate's input) */
  R rd[XMI_MAXL];    /* density x path length toward the detector point, per layer */
  int node, layer, n, h_slot; /* h_slot >= 0: exciting line of a fluorescence photon */
  long long id;
  int cfg;           /* configuration of a batched run (0 otherwise) */
  int sa_pending;    /* 1: off the solid-angle grid; the integral at (sa_r, sa_t) is still to be multiplied in */
};

/* sort key of an event: configuration, layer, interaction order */
template <typename R>
__device__ __forceinline__ int vr_key(const VrEvent<R> &ev) {
  return (ev.cfg * XMI_MAXL + ev.layer) * XMI_MAXN + ev.n - 1;
}

template <typename R>
struct VrQueue {
  VrEvent<R> *ev;
  int *key;                   /* layer * N + n - 1 */
  unsigned long long *count;
  long long cap;
};

__device__ __forceinline__ uint32_t vr_stream(int n, int sub) {
  return 0x40000000u | ((uint32_t)n << 8) | (uint32_t)sub;
}

template <typename R>
__device__ bool vr_prologue(const DevBundle<R> &b, const Photon<R> &p, const DevTally &t, VrEvent<R> &ev,
                            bool &ok) {
  if (p.E <= (R)kEnergyThreshold) return false;
  if (!XMI_CHK(p.layer, b.n_layers, 34)) { ok = false; return false; }
  const int n = p.n_int, layer = p.layer;
  /* the energy-grid location first: its gathers are in flight during the
   * geometry below (the step's atom choice reuses it) */
  locate(b, p.E, ev.node, ev.f);
  xmi_rng g;
  xmi_rng_init(&g, b.seed, (uint64_t)p.id, vr_stream(n, 0xFF));
  R radius = sqrt(uni<R>(&g)) * b.det_radius_r;
  R ang = (R)(2.0 * kPi) * uni<R>(&g);
  R dp[3] = {(R)0, cos(ang) * radius, sin(ang) * radius};
  double rel[3] = {p.c[0] - b.p_det[0], p.c[1] - b.p_det[1], p.c[2] - b.p_det[2]};
  R lcp[3];
  double total_distance;
  if constexpr (sizeof(R) == 4) {
    /* the offset from the detector is FP64 (a difference of positions), its
     * detector-frame coordinates and length FP32 */
    const float relf[3] = {(float)rel[0], (float)rel[1], (float)rel[2]};
    matvec_r(b.det_inv_r, relf, lcp);
    const float f0 = dp[0] - lcp[0], f1 = dp[1] - lcp[1], f2 = dp[2] - lcp[2];
    total_distance = sqrtf(f0 * f0 + f1 * f1 + f2 * f2);
  } else {
    double lcp_d[3];
    matvec_d(b.det_inv, rel, lcp_d);
    lcp[0] = (R)lcp_d[0], lcp[1] = (R)lcp_d[1], lcp[2] = (R)lcp_d[2];
    double e0 = (double)dp[0] - lcp_d[0], e1 = (double)dp[1] - lcp_d[1], e2 = (double)dp[2] - lcp_d[2];
    total_distance = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
  }
  R dirv[3];
  matvec_r(b.det_inv_r, p.d, dirv);
  R lcd[3] = {dp[0] - lcp[0], dp[1] - lcp[1], dp[2] - lcp[2]};
  if (lcd[0] >= (R)0) return false;
  rnorm(dirv);
  rnorm(lcd);
  R ndc[3];
  matvec_r(b.det_new_r, lcd, ndc);
  R dotprod = rdot(dirv, lcd);
  dotprod = dotprod > (R)1 ? (R)1 : (dotprod < (R)-1 ? (R)-1 : dotprod);
  const R theta = acos(dotprod);
  R proj[3];
  {
    R d = rdot(ndc, p.d);
#pragma unroll
    for (int k = 0; k < 3; k++) proj[k] = ndc[k] - d * p.d[k];
    R pn = sqrt(rdot(proj, proj));
    R ne = sqrt(rdot(p.el, p.el));
    if (pn > (R)0) {
      proj[0] /= pn; proj[1] /= pn; proj[2] /= pn;
      dotprod = (proj[0] * (p.el[0] / ne) + proj[1] * (p.el[1] / ne) + proj[2] * (p.el[2] / ne));
    } else {
      dotprod = (R)1; /* forward direction: the azimuth is undefined, take 0 */
    }
  }
  dotprod = dotprod > (R)1 ? (R)1 : (dotprod < (R)-1 ? (R)-1 : dotprod);
  const R phi = acos(dotprod);
  const R *nsam = b.n_sample_r;
  const bool up = rdot(ndc, nsam) > (R)0;

  /* path toward the detector point through the layers, as density x length */
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++) ev.rd[j] = (R)0;
  {
    PlaneWalk pw;
    if (!plane_walk_init(p.c, ndc, b.n_sample, pw, b.n_sample_r)) { ok = false; return false; }
    bool done = false, first = true;
    layers_in_direction(up, [&](int j) {
      bool active = up ? (j >= layer && j < b.n_layers) : (j <= layer);
      if (active && !done) {
        const double dd = layer_path(b, pw, j, up, first);
        if (dd > total_distance) {
          ev.rd[j] = b.rho[j] * (R)total_distance;
          done = true;
        } else {
          ev.rd[j] = b.rho[j] * (R)dd;
          total_distance = total_distance - dd;
        }
      }
    });
  }
  R murhod = (R)0;
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++) murhod += p.mus[j] * ev.rd[j];
  ev.pesc_rayl = exp(-murhod);
  R omega;
  ev.sa_pending = 0;
  if (b.use_surrogate) {
    /* the solid angle comes later from the surrogate network: the factors
     * below are stored without it, with the point's (r, theta) */
    sa_coords(b, p.c, ev.sa_r, ev.sa_t);
    omega = (R)1;
  } else {
    /* a point off the grid needs a 5000-sample integral: it is left to the
     * warp-parallel pass before the estimator (xmi_solid_angle_deferred)
     * instead of one thread of the step kernel */
    bool deferred = false;
    omega = get_solid_angle(b, p.c, p, t, ok, &deferred, &ev.sa_r, &ev.sa_t);
    ev.sa_pending = deferred ? 1 : 0;
  }
  ev.pdir_fluo = omega / (R)4 / (R)kPi;
  ev.mu_here = select_layer(p.mus, layer);
  ev.q = p.E / (R)12.39852 * sin(theta / (R)2);
  const R st = sin(theta), cp = cos(phi), ct = cos(theta);
  const R thomson = (R)1 - st * st * cp * cp;
  const R k0k = (R)1 + ((R)1 - ct) * p.E / (R)510.998928, kk0 = (R)1 / k0k;
  const R kn = (R)0.25 * kk0 * kk0 * (kk0 + k0k - (R)2 * st * st * cp * cp);
  ev.pR = omega * thomson;
  ev.pC = omega * kn;
  ev.theta = theta;
  ev.E = p.E;
  ev.w = p.w;
  ev.layer = layer;
  ev.n = n;
  ev.id = p.id;
  ev.h_slot = -1;
  if (n > 1 && p.h_type < 0) {
    if (!XMI_CHK(p.h_slot, b.n_lines, 43)) { ok = false; return false; }
    ev.h_slot = p.h_slot;
  }
  return true;
}

/* appends one event; lanes that emit together share one atomic */
template <typename R>
__device__ __forceinline__ bool vr_emit(const VrQueue<R> &q, const VrEvent<R> &ev, int key) {
  const unsigned mask = __activemask();
  const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(q.count, (unsigned long long)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  const long long i = (long long)base + __popc(mask & ((1u << lane) - 1u));
  if (i >= q.cap) return false;
  q.ev[i] = ev;
  q.key[i] = key;
  return true;
}

/* ---------------- interactions ---------------- */
template <typename R>
__device__ bool rayleigh(const DevBundle<R> &b, Photon<R> &p, xmi_rng *g) {
  bool ok = true;
  const int e = p.elem;
  const R rinv = (R)(XMI_ICDF_NR - 1), einv = (R)((XMI_ICDF_NE - 1) / (200.0 - 0.1));
  R r = uni<R>(g);
  R theta_i = bilinear(b.rayl_icdf[e], b.icdf_r, XMI_ICDF_NR, (R)0, rinv,
                       b.icdf_e, XMI_ICDF_NE, (R)0.1, einv, r, p.E, ok);
  if (!ok) return false;
  R tt = sin(theta_i) * sin(theta_i);
  tt = tt / ((R)4 - (R)2 * tt);
  r = uni<R>(g);
  R phi_i = bilinear(b.phi_icdf, b.icdf_r, XMI_ICDF_NR, (R)0, rinv, b.phi_t, XMI_PHI_NT, (R)0,
                     (R)((XMI_PHI_NT - 1) / 0.5), r, tt, ok);
  if (!ok) return false;
  R phi0 = polarisation_phi0(p);
  update_dirv(p, theta_i, phi0 + phi_i);
  update_elecv(p);
  p.h_type = XMI_RAYLEIGH;
  p.h_elem = e;
  return true;
}

/* Adv: compiled with the advanced Compton scattering (used when the bundle
 * asks for it); the default instantiation carries none of its code */
template <typename R, bool Adv = false>
__device__ bool compton(const DevBundle<R> &b, Photon<R> &p, xmi_rng *g) {
  bool ok = true;
  const int e = p.elem;
  const R rinv = (R)(XMI_ICDF_NR - 1), einv = (R)((XMI_ICDF_NE - 1) / (200.0 - 0.1));
  const R mec2 = (R)(9.10938188e-31 * 2.99792458e8 * 2.99792458e8 / 1.602176487e-19 / 1000.0);
  R r = uni<R>(g);
  R theta_i = bilinear(b.compt_icdf[e], b.icdf_r, XMI_ICDF_NR, (R)0, rinv,
                       b.icdf_e, XMI_ICDF_NE, (R)0.1, einv, r, p.E, ok);
  if (!ok) return false;
  R k0k = (R)1 + p.E * ((R)1 - cos(theta_i)) / mec2;
  R tt = sin(theta_i) * sin(theta_i);
  tt = tt / (k0k + ((R)1 / k0k) - tt) / (R)2;
  r = uni<R>(g);
  R phi_i = bilinear(b.phi_icdf, b.icdf_r, XMI_ICDF_NR, (R)0, rinv, b.phi_t, XMI_PHI_NT, (R)0,
                     (R)((XMI_PHI_NT - 1) / 0.5), r, tt, ok);
  if (!ok) return false;
  R phi0 = polarisation_phi0(p);
  if (Adv && b.use_adv_compton) {
    bool bad = false;
    p.E = (R)compton_energy_advanced(b, e, (double)p.E, (double)theta_i, g, bad);
    if (bad) return false;
    if (p.E == (R)0) return true;
    mu_calc(b, p.E, p.mus);
  } else {
    p.E = compton_energy(b, e, p.E, theta_i, g, false, ok);
    if (!ok) return false;
    mu_calc(b, p.E, p.mus);
    if (p.E == (R)0) return true;
  }
  update_dirv(p, theta_i, phi_i + phi0);
  update_elecv(p);
  R cti = cos(theta_i), cpi = cos(phi_i), spi = sin(phi_i);
  R pp = (R)2 * ((cti * cpi) * (cti * cpi) + spi * spi);
  R rat = (R)1 / ((R)1 + ((R)1 - cti) * p.E / (R)(double)510.998910f);
  R rk = rat - (R)2 + (R)1 / rat;
  pp = pp / (rk + pp);
  r = uni<R>(g);
  R w_h = ((R)1 + pp) / (R)2;
  if (r > w_h) {
    R c0 = p.d[1] * p.el[2] - p.d[2] * p.el[1];
    R c1 = p.d[2] * p.el[0] - p.d[0] * p.el[2];
    R c2 = p.d[0] * p.el[1] - p.d[1] * p.el[0];
    p.el[0] = c0; p.el[1] = c1; p.el[2] = c2;
  }
  p.h_type = XMI_COMPTON;
  p.h_elem = e;
  return true;
}

/* xmi_coster_kronig_check (src/xmi_main.F90:5184-5323) */
template <typename R>
__device__ __forceinline__ int coster_kronig(const R *ck, int shell, xmi_rng *g) {
  for (int guard = 0; guard < 16; guard++) {
    R r, s;
    switch (shell) {
      case 2:
        r = uni<R>(g);
        return r < __ldg(ck + XMI_FL23) ? 3 : 2;
      case 1:
        r = uni<R>(g);
        s = __ldg(ck + XMI_FL12);
        if (r < s) { shell = 2; continue; }
        s += __ldg(ck + XMI_FL13);
        return r < s ? 3 : 1;
      case 7:
        r = uni<R>(g);
        return r < __ldg(ck + XMI_FM45) ? 8 : 7;
      case 6:
        r = uni<R>(g);
        s = __ldg(ck + XMI_FM34);
        if (r < s) { shell = 7; continue; }
        s += __ldg(ck + XMI_FM35);
        return r < s ? 8 : 6;
      case 5:
        r = uni<R>(g);
        s = __ldg(ck + XMI_FM23);
        if (r < s) { shell = 6; continue; }
        s += __ldg(ck + XMI_FM24);
        if (r < s) { shell = 7; continue; }
        s += __ldg(ck + XMI_FM25);
        return r < s ? 8 : 5;
      case 4:
        r = uni<R>(g);
        s = __ldg(ck + XMI_FM12);
        if (r < s) { shell = 5; continue; }
        s += __ldg(ck + XMI_FM13);
        if (r < s) { shell = 6; continue; }
        s += __ldg(ck + XMI_FM14);
        if (r < s) { shell = 7; continue; }
        s += __ldg(ck + XMI_FM15);
        return r < s ? 8 : 4;
      default:
        return shell;
    }
  }
  return shell;
}

/* ---------------- analog cascades (VR off), src/xmi_main.F90:2413-4783 ----------------
 * A photon simulates at most one cascade; its offspring (at most one) takes
 * the photon's state at the interaction, draws from the streams of
 * id | kOffspringId and simulates no cascade of its own. */
constexpr long long kOffspringId = 1ll << 62;

/* The photon of a vacancy in shell s (1..8 = L1..M5) of element e, set up as
 * the cascade routines set up their photons (src/xmi_main.F90:4696-4760):
 * the cascade-corrected yield, Coster-Kronig, the line, an isotropic
 * direction and a random E-vector perpendicular to it.  True when a line
 * above the threshold is emitted.  Shells beyond M5 emit nothing (no lines;
 * the reference reads past its 9-shell yield table for them). */
template <typename R>
__device__ __noinline__ bool cascade_photon(const DevBundle<R> &b, int e, int s, Photon<R> &q, xmi_rng *g) {
  if (s < 1 || s > 8) return false;
  if (s >= 4 && !b.use_M_lines) return false;
  R r = uni<R>(g);
  if (r > XMI_LDG(b.yield_corr, (long long)e * XMI_NSHELL + s, (long long)b.n_elem * XMI_NSHELL, 15)) return false;
  s = coster_kronig(b.ck + (size_t)e * XMI_NCK, s, g);
  r = uni<R>(g);
  R sumz = (R)0;
  int slot = -1;
  const int s0 = XMI_LDG(b.shell_off, 10 * e + s, 10 * b.n_elem, 16);
  const int s1 = XMI_LDG(b.shell_off, 10 * e + s + 1, 10 * b.n_elem, 16);
  for (int sl = s0; sl < s1; sl++) {
    sumz = sumz + XMI_LDG(b.line_rate, sl, b.n_lines, 17);
    if (r < sumz) { slot = sl; break; }
  }
  if (slot < 0) return false;
  const R E = XMI_LDG(b.line_energy, slot, b.n_lines, 17);
  if (E <= (R)kEnergyThreshold) return false;
  q.E = E;
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++)
    q.mus[j] = j < b.n_layers ? XMI_LDG(b.precalc_mu, (long long)j * b.n_lines + slot,
                                        (long long)b.n_layers * b.n_lines, 18) : (R)0;
  q.theta = acos((R)2 * uni<R>(g) - (R)1);
  q.phi = (R)(2.0 * kPi) * uni<R>(g);
  q.d[0] = sin(q.theta) * cos(q.phi);
  q.d[1] = sin(q.theta) * sin(q.phi);
  q.d[2] = cos(q.theta);
  const R rr = (R)(2.0 * kPi) * uni<R>(g);
  q.el[0] = cos(rr);
  q.el[1] = sin(rr);
  q.el[2] = (R)0;
  const R cosalfa = q.el[0] * q.d[0] + q.el[1] * q.d[1] + q.el[2] * q.d[2];
  if (fabs(cosalfa) > (R)1) return false; /* the reference stops the program here */
  const R c_ae = (R)1 / sin(acos(cosalfa)), c_be = -c_ae * cosalfa;
#pragma unroll
  for (int k = 0; k < 3; k++) q.el[k] = c_ae * q.el[k] + c_be * q.d[k];
  q.h_type = -XMI_LDG(b.line_index, slot, b.n_lines, 17);
  q.h_elem = e;
  q.h_slot = slot;
  q.last = XMI_PHOTOELECTRIC;
  return true;
}

/* the offspring of photon p: its state at the interaction, its own streams */
template <typename R>
__device__ __forceinline__ void offspring_from(const Photon<R> &p, Photon<R> &q) {
  q = p;
  q.id = p.id | kOffspringId;
  q.hit = 0;
  q.inside = 0;
}

/* cascade flags of the photo-absorption kernel: in kCascAllowed (this photon
 * may still cascade), out kCascUsed (its cascade happened) and kCascChild
 * (an offspring was made) */
enum : int { kCascAllowed = 1, kCascUsed = 2, kCascChild = 4 };

/* xmi_simulate_photon_cascade_auger (src/xmi_main.F90:2413-4594): a K/L
 * vacancy decayed without a photon (p's energy is already 0); the
 * transition's first vacancy turns p into its fluorescence photon, the second
 * gives the offspring */
template <typename R>
__device__ __noinline__ void cascade_auger(const DevBundle<R> &b, Photon<R> &p, int shell, Photon<R> &child,
                                           int &flags, xmi_rng *g) {
  const int e = p.elem, nt = shell == 0 ? XMI_AUGER_K : XMI_AUGER_L, nb = shell == 0 ? 30 : 27;
  const int f0 = shell == 0 ? 1 : 4;
  const long long base = ((long long)e * 4 + shell) * XMI_AUGER_K, lim = (long long)b.n_elem * 4 * XMI_AUGER_K;
  const R r = uni<R>(g);
  R sumz = (R)0;
  int t = -1;
  for (int k = 0; k < nt; k++) {
    sumz = sumz + XMI_LDG(b.auger_rate, base + k, lim, 52);
    if (r < sumz) { t = k; break; }
  }
  if (t < 0) return;
  offspring_from(p, child);
  if (cascade_photon(b, e, f0 + t / nb, p, g)) flags |= kCascUsed;
  if (cascade_photon(b, e, f0 + t % nb, child, g)) flags |= kCascChild;
}

/* Casc: compiled with the analog cascades; child receives the offspring and
 * flags carries kCasc* */
template <typename R, bool Casc = false>
__device__ bool fluorescence(const DevBundle<R> &b, Photon<R> &p, xmi_rng *g, Photon<R> *child = nullptr,
                             int *flags = nullptr) {
  const int e = p.elem;
  int node;
  R f;
  locate(b, p.E, node, f);
  R photo_total = el_val(b, e, XMI_REC_PHOTO, node, f);
  R sumz = (R)0, r = uni<R>(g);
  int shell = -1;
  if constexpr (sizeof(R) == 4) {
    /* r < sum of partial / total, as r total < sum of partials: no division
     * per shell */
    const R target = r * photo_total;
    for (int s = 0; s <= b.max_shell; s++) {
      sumz = sumz + el_val(b, e, XMI_REC_PART + s, node, f);
      if (target < sumz) { shell = s; break; }
    }
  } else {
    for (int s = 0; s <= b.max_shell; s++) {
      sumz = sumz + el_val(b, e, XMI_REC_PART + s, node, f) / photo_total;
      if (r < sumz) { shell = s; break; }
    }
  }
  if (shell < 0) {
    p.E = (R)0;
    return true;
  }
  const R yc = XMI_LDG(b.yield_corr, (long long)e * XMI_NSHELL + shell, (long long)b.n_elem * XMI_NSHELL, 15);
  if (b.use_vr == 0 && b.escape_mode == 0) {
    r = uni<R>(g);
    if (r > yc) {
      p.E = (R)0;
      if constexpr (Casc) {
        if ((*flags & kCascAllowed) && b.casc_auger && shell <= 3) cascade_auger(b, p, shell, *child, *flags, g);
      }
      return true;
    }
  } else {
    (void)uni<R>(g);
    if (b.escape_mode) p.we = p.we * yc;
    else p.w = p.w * yc;
  }
  shell = coster_kronig(b.ck + (size_t)e * XMI_NCK, shell, g);
  r = uni<R>(g);
  sumz = (R)0;
  int slot = -1;
  const int s0 = XMI_LDG(b.shell_off, 10 * e + shell, 10 * b.n_elem, 16);
  const int s1 = XMI_LDG(b.shell_off, 10 * e + shell + 1, 10 * b.n_elem, 16);
  for (int sl = s0; sl < s1; sl++) {
    sumz = sumz + XMI_LDG(b.line_rate, sl, b.n_lines, 17);
    if (r < sumz) { slot = sl; break; }
  }
  if (slot < 0) {
    p.E = (R)0;
    return true;
  }
  p.E = XMI_LDG(b.line_energy, slot, b.n_lines, 17);
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++)
    p.mus[j] = j < b.n_layers ? XMI_LDG(b.precalc_mu, (long long)j * b.n_lines + slot,
                                        (long long)b.n_layers * b.n_lines, 18) : (R)0;
  R theta_i = acos((R)-2 * uni<R>(g) + (R)1);
  R phi_i = (R)(2.0 * kPi) * uni<R>(g);
  update_dirv(p, theta_i, phi_i);
  update_elecv(p);
  p.h_type = -XMI_LDG(b.line_index, slot, b.n_lines, 17);
  p.h_elem = e;
  p.h_slot = slot;
  if constexpr (Casc) {
    /* xmi_simulate_photon_cascade_radiative, src/xmi_main.F90:4596-4783 */
    const int u = XMI_LDG(b.line_casc, slot, b.n_lines, 53);
    if ((*flags & kCascAllowed) && b.casc_rad && u >= 0) {
      offspring_from(p, *child);
      if (cascade_photon(b, e, u, *child, g)) *flags |= kCascUsed | kCascChild;
    }
  }
  return true;
}

/* ---------------- analog detector checks ---------------- */
/* xmi_check_detector_intersection (src/xmi_aux_f.F90:1622-1834), including
 * the reference's use of the scalar segment length as the direction of the
 * collimator-free branch; evaluated in FP64 */
__device__ inline int check_detector_intersection(const double *p_det, const double *det_inv, int coll_present,
                                           double det_radius, double coll_height, double half_apex,
                                           double vx, const double *bc, const double *ec) {
  double t0[3] = {bc[0] - p_det[0], bc[1] - p_det[1], bc[2] - p_det[2]};
  double t1[3] = {ec[0] - p_det[0], ec[1] - p_det[1], ec[2] - p_det[2]};
  double bd[3], ed[3];
  matvec_d(det_inv, t0, bd);
  matvec_d(det_inv, t1, ed);
  if (!coll_present) {
    if (bd[0] * ed[0] > 0) return 0;
    double s = sqrt((ed[0] - bd[0]) * (ed[0] - bd[0]) + (ed[1] - bd[1]) * (ed[1] - bd[1]) + (ed[2] - bd[2]) * (ed[2] - bd[2]));
    if (s == 0.0) return 3;
    double d = (0.0 - ed[0]) / s;
    double iy = d * s + ed[1], iz = d * s + ed[2];
    if (sqrt(iy * iy + iz * iz) <= det_radius) return 3; /* direction component along x is s >= 0 */
    return 0;
  }
  double dv[3] = {ed[0] - bd[0], ed[1] - bd[1], ed[2] - bd[2]};
  double tb = (bd[0] - ed[0]) / dv[0], te = (ed[0] - ed[0]) / dv[0];
  double delta[3] = {ed[0] - vx, ed[1], ed[2]};
  double cos2t = cos(half_apex) * cos(half_apex);
  double c2 = dv[0] * (1.0 - cos2t) * dv[0] - dv[1] * cos2t * dv[1] - dv[2] * cos2t * dv[2];
  double c1 = dv[0] * (1.0 - cos2t) * delta[0] - dv[1] * cos2t * delta[1] - dv[2] * cos2t * delta[2];
  double c0 = delta[0] * (1.0 - cos2t) * delta[0] - delta[1] * cos2t * delta[1] - delta[2] * cos2t * delta[2];
  double disc = c1 * c1 - c0 * c2;
  if (disc < 0.0) return 0;
  double tt1 = (-c1 + sqrt(disc)) / c2, tt2 = (-c1 - sqrt(disc)) / c2;
  double X1x = ed[0] + tt1 * dv[0], X2x = ed[0] + tt2 * dv[0];
  int nvalid = 0;
  if (-(X1x - vx) >= 0.0) nvalid = 1;
  if (-(X2x - vx) >= 0.0) nvalid = (nvalid == 1) ? 3 : 2;
  double tmax = tb > te ? tb : te, tmin = tb < te ? tb : te;
  if (nvalid == 0) return 0;
  if (nvalid == 3) {
    if (tt1 <= tmax && tt1 >= tmin && X1x <= coll_height) return 1;
    if (tt2 <= tmax && tt2 >= tmin && X2x <= coll_height) return 1;
    return 0;
  }
  double tsel = nvalid == 1 ? tt1 : tt2, Xsx = nvalid == 1 ? X1x : X2x;
  if (tsel <= tmax && tsel >= tmin && Xsx <= coll_height) return 1;
  if (dv[0] == 0.0) return 3;
  double d = (0.0 - ed[0]) / dv[0];
  double iy = d * dv[1] + ed[1], iz = d * dv[2] + ed[2];
  double db = sqrt(bd[0] * bd[0] + (bd[1] - iy) * (bd[1] - iy) + (bd[2] - iz) * (bd[2] - iz));
  double de = sqrt((bd[0] - ed[0]) * (bd[0] - ed[0]) + (bd[1] - ed[1]) * (bd[1] - ed[1]) + (bd[2] - ed[2]) * (bd[2] - ed[2]));
  if (sqrt(iy * iy + iz * iz) <= det_radius && db <= de) {
    if (dv[0] >= 0.0) return 3;
    return 2;
  }
  return 0;
}

/* xmi_check_photon_detector_hit (src/xmi_main.F90:1920-1984) */
template <typename R>
__device__ bool check_photon_detector_hit(const DevBundle<R> &b, const Photon<R> &p) {
  double dvd[3] = {(double)p.d[0], (double)p.d[1], (double)p.d[2]};
  if (dot3(dvd, b.n_det) >= 0.0) return false;
  double dd[3], cd[3], t[3] = {p.c[0] - b.p_det[0], p.c[1] - b.p_det[1], p.c[2] - b.p_det[2]};
  matvec_d(b.det_inv, dvd, dd);
  matvec_d(b.det_inv, t, cd);
  if (dd[0] == 0.0) return false;
  double s = (0.0 - cd[0]) / dd[0];
  double iy = s * dd[1] + cd[1], iz = s * dd[2] + cd[2];
  if (sqrt(iy * iy + iz * iz) > b.det_radius) return false;
  if (!b.coll_present) return true;
  s = (b.coll_height - cd[0]) / dd[0];
  iy = s * dd[1] + cd[1];
  iz = s * dd[2] + cd[2];
  return sqrt(iy * iy + iz * iz) <= b.coll_radius;
}

/* ---------------- one history ---------------- */
enum StepStatus { kStepDone = 0, kStepInteract = 1, kStepError = 2 };

/* One step of a photon (one pass of the loop of xmi_simulate_photon,
 * src/xmi_main.F90:1188-1685): transport to the next interaction point
 * (forced with variance reduction, analog otherwise), the estimator event of
 * that interaction, and the choice of atom and interaction type (p.elem,
 * p.last).  Returns kStepInteract with g positioned on the draws of the
 * interaction, or kStepDone when the history ends (p.hit marks a detector
 * hit), or kStepError. */
template <typename R>
__device__ int step_photon(const DevBundle<R> &b, Photon<R> &p, const DevTally &t, const VrQueue<R> &vq, int cfg,
                           xmi_rng &g) {
  if (p.E < (R)kEnergyThreshold) return kStepDone;
  p.inside = 0;
  xmi_rng_init(&g, b.seed, (uint64_t)p.id, (uint32_t)(p.n_int + 1));
  const R *dn = b.n_sample_r;
  const bool up = rdot(p.d, dn) > (R)0;
  const R R0 = uni<R>(&g);
  if ((b.escape_mode == 1 && p.n_int == 1) || (b.use_vr == 0 && b.escape_mode == 0)) {
    R minr = (R)0, maxr = (R)0, blbs = (R)1;
    bool stop = false;
    int outcome = 0; /* 0 continue, 1 photon absorbed by collimator/bad hit, 2 detector hit, 3 error */
    PlaneWalk pw;
    if (!plane_walk_init(p.c, p.d, b.n_sample, pw, b.n_sample_r)) return kStepError;
    layers_in_direction(up, [&](int j) {
      bool active = up ? (j >= p.layer && j < b.n_layers) : (j <= p.layer);
      if (!active || stop) return;
      const double sw = plane_walk(pw, up ? b.zend[j] : b.zbeg[j], b.n_sample);
      const double dd = fabs(sw) * pw.dlen;
      double ip[3];
#pragma unroll
      for (int q = 0; q < 3; q++) ip[q] = sw * (double)p.d[q] + p.c[q];
      /* FP32: the step's 1/cos is FP32, so the crossing point's height is
       * set to the plane's exactly (see the forced step below) */
      if constexpr (sizeof(R) == 4) set_height(ip, b.n_sample, (up ? b.zend[j] : b.zbeg[j]) * b.n_sample[2]);
      R tp = (R)-1 * (R)dd * b.rho[j] * p.mus[j];
      R tempexp = exp(tp);
      minr = maxr;
      maxr = maxr - blbs * expm1(tp);
      if (R0 <= maxr) {
        R dist = (R)-1 * log1p((R)-1 * (R0 - minr) / blbs) / p.mus[j] / b.rho[j];
        double tc[3] = {p.c[0], p.c[1], p.c[2]};
#pragma unroll
        for (int q = 0; q < 3; q++) p.c[q] = p.c[q] + (double)dist * (double)p.d[q];
        if (b.escape_mode != 1) {
          int rc = check_detector_intersection(b.p_det, b.det_inv, b.coll_present, b.det_radius, b.coll_height,
                                               b.coll_half_apex, b.coll_vertex_x, tc, p.c);
          if (rc == 1 || rc == 3) { outcome = 1; stop = true; return; }
          if (rc == 2) { outcome = 2; stop = true; return; }
        }
        p.layer = j;
        p.inside = 1;
        stop = true;
      } else {
        if (b.escape_mode != 1) {
          int rc = check_detector_intersection(b.p_det, b.det_inv, b.coll_present, b.det_radius, b.coll_height,
                                               b.coll_half_apex, b.coll_vertex_x, p.c, ip);
          if (rc == 1 || rc == 3) { outcome = 1; stop = true; return; }
          if (rc == 2) { outcome = 2; stop = true; return; }
        }
        p.c[0] = ip[0]; p.c[1] = ip[1]; p.c[2] = ip[2];
        blbs = blbs * tempexp;
      }
    });
    if (outcome == 3) return kStepError;
    if (outcome == 1) return kStepDone;
    if (outcome == 2) { p.hit = 1; return kStepDone; }
  } else {
    if (p.n_int == b.N) return kStepDone;
    R dist[XMI_MAXL];
    R pabs = (R)0;
    const int cur = p.layer;
    PlaneWalk pw;
    if (!plane_walk_init(p.c, p.d, b.n_sample, pw, b.n_sample_r)) return kStepError;
    bool first = true;
    layers_in_direction(up, [&](int j) {
      bool active = up ? (j >= cur && j < b.n_layers) : (j <= cur);
      dist[j] = (R)0;
      if (active) {
        dist[j] = (R)layer_path(b, pw, j, up, first);
        pabs = pabs + p.mus[j] * b.rho[j] * dist[j];
      }
    });
    R pabs2 = (R)-1 * expm1((R)-1 * pabs);
    p.w = p.w * pabs2;
    if (b.escape_mode == 1) p.we = p.w;
    R negln = (R)-1 * log1p((R)-1 * R0 * pabs2);
    int my_index = cur;
    R my_sum = (R)0, sum_before = (R)0;
    bool found = false;
    layers_in_direction(up, [&](int j) {
      bool active = up ? (j >= cur && j < b.n_layers) : (j <= cur);
      if (active && !found) {
        const R prev = my_sum;
        my_sum = my_sum + p.mus[j] * b.rho[j] * dist[j];
        if (my_sum > negln) { my_index = j; found = true; sum_before = prev; }
      }
    });
    R mr_sel = (R)0;
#pragma unroll
    for (int j = 0; j < XMI_MAXL; j++)
      if (j == my_index) mr_sel = p.mus[j] * b.rho[j];
    R temp_sum = (R)0;
    layers_in_direction(up, [&](int j) {
      bool active = up ? (j >= cur && j <= my_index) : (j <= cur && j >= my_index);
      if (active) temp_sum = temp_sum + ((R)1 - (p.mus[j] * b.rho[j] / mr_sel)) * dist[j];
    });
    temp_sum = temp_sum - (R)1 * log1p((R)-1 * R0 * pabs2) / mr_sel;
    if (!XMI_CHK(my_index, b.n_layers, 41)) return kStepError;
    const double h0 = pw.h;
#pragma unroll
    for (int q = 0; q < 3; q++) p.c[q] = p.c[q] + (double)temp_sum * (double)p.d[q];
    if constexpr (sizeof(R) == 4) {
      /* FP32: after centimetres of air the step's rounding is a few nm, the
       * same for every photon of a pencil beam -- a systematic shift of all
       * interaction depths, which biased lines absorbed within ~0.1 um of a
       * surface (Au M lines: -2% behind 5 cm of air).  The height along the
       * normal, which every escape path depends on, is therefore set in FP64:
       * the entry plane of the selected layer (or the current height when
       * the photon stays in its layer) plus the depth into that layer. */
      const R into = (negln - (found ? sum_before : (R)0)) / mr_sel;
      const double h_in = (my_index == cur || !found) ? h0 : (up ? b.zbeg[my_index] : b.zend[my_index]) * b.n_sample[2];
      const double hb = b.zbeg[my_index] * b.n_sample[2], he = b.zend[my_index] * b.n_sample[2];
      double h = h_in + (double)(into * rdot(p.d, b.n_sample_r));
      h = h < hb ? hb : (h > he ? he : h);
      set_height(p.c, b.n_sample, h);
    }
    p.inside = 1;
    p.layer = my_index;
  }
  if (!p.inside) {
    if (b.escape_mode != 1) p.hit = check_photon_detector_hit(b, p) ? 1 : 0;
    return kStepDone;
  }
  if (p.n_int == b.N) return kStepDone;
  p.n_int = p.n_int + 1;
  int node = -1; /* energy-grid location of p.E: from the event when there is one */
  R f = (R)0;
  if (b.use_vr == 1) {
    bool ok = true;
    VrEvent<R> ev;
    ev.cfg = cfg;
    if (vr_prologue(b, p, t, ev, ok)) {
      node = ev.node;
      f = ev.f;
      if (!vr_emit(vq, ev, vr_key(ev))) { set_error(t, kErrQueue); return kStepError; }
    }
    if (!ok) { set_error(t, kErrTable); return kStepError; }
  }
  /* atom selection and interaction type, src/xmi_main.F90:1556-1652 */
  if (node < 0) locate(b, p.E, node, f);
  R r = uni<R>(&g);
  if (!XMI_CHK(p.layer, b.n_layers, 33)) return kStepError;
  const int L = p.layer, nel = b.nel[L], off = b.off[L];
  R mu_l = (R)0;
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++)
    if (j == L) mu_l = p.mus[j];
  int sel = nel - 1;
  if constexpr (sizeof(R) == 4) {
    /* the same choice, r < sum_k<=i w_k sigma_k(E) / mu, as r mu < the
     * layer's running sum at E: the running sums interpolate linearly like
     * each term, and a node's sums are one contiguous row instead of one
     * element record (a dependent gather) per term */
    const long long c0 = (long long)node * b.n_layer_el + off, lim = (long long)b.n_nodes * b.n_layer_el;
    const R target = r * mu_l;
    for (int i = 0; i < nel; i++) {
      const R v0 = XMI_LDG(b.layer_cs, c0 + i, lim, 60), v1 = XMI_LDG(b.layer_cs, c0 + b.n_layer_el + i, lim, 60);
      if (target < v0 + f * (v1 - v0)) { sel = i; break; }
    }
  } else {
    R thr = (R)0;
    for (int i = 0; i < nel; i++) {
      thr = thr + XMI_LDG(b.layer_w, off + i, b.n_layer_el, 19) *
                      el_val(b, XMI_LDG(b.layer_el, off + i, b.n_layer_el, 19), XMI_REC_TOT, node, f) / mu_l;
      if (r < thr) { sel = i; break; }
    }
  }
  p.elem = XMI_LDG(b.layer_el, off + sel, b.n_layer_el, 19);
  if (!XMI_CHK(p.elem, b.n_elem, 42)) return kStepError;
  r = uni<R>(&g);
  R pr = el_val(b, p.elem, XMI_REC_PR, node, f);
  R prc = el_val(b, p.elem, XMI_REC_PRC, node, f);
  p.last = r < pr ? XMI_RAYLEIGH : (r < prc ? XMI_COMPTON : XMI_PHOTOELECTRIC);
  return kStepInteract;
}

/* the interaction chosen by step_photon, drawing from g */
template <typename R, bool Adv = false>
__device__ __forceinline__ bool interact(const DevBundle<R> &b, Photon<R> &p, const DevTally &t, xmi_rng &g) {
  bool ok;
  if (p.last == XMI_RAYLEIGH) ok = rayleigh(b, p, &g);
  else if (p.last == XMI_COMPTON) ok = compton<R, Adv>(b, p, &g);
  else ok = fluorescence(b, p, &g);
  if (!ok) set_error(t, kErrTable);
  return ok;
}

/* a whole history in one thread: false on an error (no tally) */
template <typename R>
__device__ bool simulate_photon(const DevBundle<R> &b, Photon<R> &p, const DevTally &t, const VrQueue<R> &vq,
                                int cfg) {
  for (int guard = 0; guard < 4 * XMI_MAXN + 8; guard++) {
    xmi_rng g;
    const int st = step_photon(b, p, t, vq, cfg, g);
    if (st == kStepDone) return true;
    if (st == kStepError) return false;
    if (!interact(b, p, t, g)) return false;
  }
  return true;
}

/* ---------------- source sampling (src/xmi_main.F90:319-858) ---------------- */
template <typename R>
__device__ __forceinline__ R ran_gauss(xmi_rng *g, R sigma) {
  if constexpr (sizeof(R) == 4) {
    /* Box-Muller in FP32 on the same two draws */
    float u1 = uni<float>(g);
    const float u2 = uni<float>(g);
    if (u1 <= 0.0f) u1 = 0x1p-25f;
    return sigma * sqrtf(-2.0f * logf(u1)) * cosf((float)(2.0 * kPi) * u2);
  } else {
    double u1 = xmi_rng_uniform(g), u2 = xmi_rng_uniform(g);
    if (u1 <= 0.0) u1 = 1.0 / 9007199254740992.0;
    return (R)(sigma * sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2));
  }
}

/* FP32 source sampling of one photon (energy, weight, direction, position on
 * the first layer's entry plane): the same draws and distributions as the
 * FP64 path below, without FP64 arithmetic except the position.
 * The trapezoid's inverse CDF is the root t = E - x1 of
 * m/2 t^2 + y1 t - area u = 0 in [0, x2 - x1] (xmi_ran_trap), written as
 * 2 area u / (y1 + sqrt(y1^2 + 2 m area u)), which does not cancel. */
__device__ __forceinline__ bool start_photon_f32(const DevBundle<float> &b, const xmi_source_item &it, long long j, Photon<float> &p,
                                 bool &skip) {
  xmi_rng g;
  xmi_rng_init(&g, b.seed, (uint64_t)p.id, 0u);
  skip = false;
  const ItemF &f = b.items_f[&it - b.items];
  float hvr = 0.0f;
  if (it.kind == 0) {
    const float du = f.area * uni<float>(&g);
    const float disc = fmaxf(fmaf(2.0f * f.m, du, f.y1 * f.y1), 0.0f);
    const float den = f.y1 + sqrtf(disc);
    float t = den > 0.0f ? 2.0f * du / den : 0.0f;
    t = fminf(fmaxf(t, 0.0f), f.de);
    p.E = f.e0 + t;
    const float fr = t * f.inv_de;
    hvr = fmaf(f.dh, fr, f.h0) / fmaf(f.di, fr, f.i0);
    int node;
    float fl;
    locate(b, p.E, node, fl);
    const float ex0 = XMI_LDG(b.exc_tab, node, b.n_nodes, 20), ex1 = XMI_LDG(b.exc_tab, node + 1, b.n_nodes, 20);
    const float exc_corr = expf(-(ex0 + fl * (ex1 - ex0)));
    mu_calc(b, p.E, p.mus);
    p.w = f.weight * exc_corr;
  } else {
    if (it.dist_type == 1) {
      p.E = ran_gauss<float>(&g, f.scale) + f.e0;
      if (p.E <= (float)kEnergyThreshold || p.E > (float)kEnergyMax) { skip = true; return true; }
    } else if (it.dist_type == 2) {
      float u;
      do { u = uni<float>(&g); } while (u == 0.5f);
      p.E = f.scale * tanf((float)kPi * u) + f.e0;
      if (!(p.E > (float)kEnergyThreshold && p.E <= (float)kEnergyMax)) { skip = true; return true; }
    } else {
      p.E = f.e0;
    }
    mu_calc(b, p.E, p.mus);
    p.w = f.weight;
  }
  /* xmi_coords_dir */
  float x1, y1;
  double h = 0.0;
  if (!f.gauss) {
    x1 = b.slit_ax_r * fmaf(2.0f, uni<float>(&g), -1.0f);
    y1 = b.slit_ay_r * fmaf(2.0f, uni<float>(&g), -1.0f);
    p.c[0] = p.c[1] = p.c[2] = 0.0;
  } else {
    x1 = ran_gauss<float>(&g, (float)it.sigma_xp);
    y1 = ran_gauss<float>(&g, (float)it.sigma_yp);
    p.c[0] = (double)(ran_gauss<float>(&g, (float)it.sigma_x) - b.d_source_slit_r * sinf(x1));
    p.c[1] = (double)(ran_gauss<float>(&g, (float)it.sigma_y) - b.d_source_slit_r * sinf(y1));
    p.c[2] = 0.0;
    h = p.c[0] * b.n_sample[0] + p.c[1] * b.n_sample[1];
  }
  const float dx = tanf(x1), dy = tanf(y1), inv = 1.0f / sqrtf(dx * dx + dy * dy + 1.0f);
  p.d[0] = dx * inv; p.d[1] = dy * inv; p.d[2] = inv;
  p.theta = acosf(p.d[2]);
  p.phi = atan2f(p.d[1], p.d[0]);
  bool horizontal;
  if (it.kind == 0) horizontal = uni<float>(&g) <= hvr;
  else horizontal = (double)(it.local0 + j + 1) <= it.hor_ver_ratio;
  if (horizontal) { p.el[0] = 0.0f; p.el[1] = 1.0f; p.el[2] = 0.0f; }
  else { p.el[0] = 1.0f; p.el[1] = 0.0f; p.el[2] = 0.0f; }
  p.we = p.w;
  const float cosalfa = rdot(p.el, p.d);
  if (fabsf(cosalfa) > 1.0f) return false;
  const float c_ae = 1.0f / sinf(acosf(cosalfa)), c_be = -c_ae * cosalfa;
#pragma unroll
  for (int k = 0; k < 3; k++) p.el[k] = c_ae * p.el[k] + c_be * p.d[k];
  /* xmi_photon_shift_first_layer: the source lies before the first layer
   * (zbeg[0] > 0 after xmi_init_input), so the photon moves onto its entry
   * plane; the step's 1/cos is FP32 (the lateral position is off by ~1e-7
   * of the source distance) and the height is set to the plane's in FP64 */
  p.layer = -1;
  if (p.c[2] >= b.zbeg[0]) {
    for (int i = 0; i < b.n_layers; i++)
      if (p.c[2] < b.zend[i]) { p.layer = i; break; }
    if (p.layer < 0) return false;
  } else {
    const float itn = rdot(p.d, b.n_sample_r);
    if (itn == 0.0f) return false;
    const float sw = (float)(b.hbeg0 - h) / itn;
#pragma unroll
    for (int k = 0; k < 3; k++) p.c[k] += (double)(sw * p.d[k]);
    set_height(p.c, b.n_sample, b.hbeg0);
    p.layer = 0;
  }
  return true;
}

template <typename R>
__device__ bool start_photon(const DevBundle<R> &b, const xmi_source_item &it, long long j, Photon<R> &p,
                             bool &skip) {
  xmi_rng g;
  xmi_rng_init(&g, b.seed, (uint64_t)p.id, 0u);
  skip = false;
  double hvr = 0.0;
  if (it.kind == 0) {
    /* xmi_ran_trap + xmi_poly_solve_quadratic */
    double m = it.trap[1], denom = it.trap[0], x1 = it.trap[2], x2 = it.trap[3], y1 = it.trap[4];
    double a = m / 2.0, bq = y1 - x1 * m, c = -x1 * y1 + m * x1 * x1 / 2.0 - denom * xmi_rng_uniform(&g);
    double E;
    if (a == 0.0) {
      if (bq == 0.0) return false;
      E = -1.0 * c / bq;
      if (!(x1 <= E && E <= x2)) return false;
    } else {
      double delta = bq * bq - 4.0 * a * c;
      if (delta < 0.0) return false;
      double sd = sqrt(delta), t1 = (-bq + sd) / 2.0 / a, t2 = (-bq - sd) / 2.0 / a;
      double r1 = t1 < t2 ? t1 : t2, r2 = t1 > t2 ? t1 : t2;
      if (x1 <= r1 && r1 <= x2) E = r1;
      else if (x1 <= r2 && r2 <= x2) E = r2;
      else return false;
    }
    p.E = (R)E;
    hvr = (it.h0 + ((it.h1 - it.h0) * (E - it.e0) / (it.e1 - it.e0))) /
          (it.i0 + ((it.i1 - it.i0) * (E - it.e0) / (it.e1 - it.e0)));
    int node;
    R f;
    locate(b, p.E, node, f);
    R ex0 = XMI_LDG(b.exc_tab, node, b.n_nodes, 20), ex1 = XMI_LDG(b.exc_tab, node + 1, b.n_nodes, 20);
    R exc_corr = exp((R)-1 * (ex0 + f * (ex1 - ex0)));
    mu_calc(b, p.E, p.mus);
    p.w = (R)it.weight * exc_corr;
  } else {
    if (it.dist_type == 1) {
      p.E = ran_gauss<R>(&g, (R)it.scale) + (R)it.e0;
      if (p.E <= (R)kEnergyThreshold || p.E > (R)kEnergyMax) { skip = true; return true; }
    } else if (it.dist_type == 2) {
      double u;
      do { u = xmi_rng_uniform(&g); } while (u == 0.5);
      p.E = (R)(it.scale * tan(kPi * u) + it.e0);
      if (p.E <= (R)kEnergyThreshold || p.E > (R)kEnergyMax) { skip = true; return true; }
    } else {
      p.E = (R)it.e0;
    }
    mu_calc(b, p.E, p.mus);
    p.w = (R)it.weight;
  }
  /* xmi_coords_dir */
  double x1, y1;
  if (fabs(it.sigma_x * it.sigma_y) < (double)1.0e-20f) {
    /* atan(slit / d_source_slit / 2), a constant of the run computed once on the host */
    const double x1m = b.slit_ax, y1m = b.slit_ay;
    double u = xmi_rng_uniform(&g);
    x1 = x1m * (-1.0 * (1.0 - u) + 1.0 * u);
    u = xmi_rng_uniform(&g);
    y1 = y1m * (-1.0 * (1.0 - u) + 1.0 * u);
    p.c[0] = p.c[1] = p.c[2] = 0.0;
  } else {
    x1 = ran_gauss<double>(&g, it.sigma_xp);
    y1 = ran_gauss<double>(&g, it.sigma_yp);
    p.c[0] = ran_gauss<double>(&g, it.sigma_x) - b.d_source_slit * sin(x1);
    p.c[1] = ran_gauss<double>(&g, it.sigma_y) - b.d_source_slit * sin(y1);
    p.c[2] = 0.0;
  }
  if constexpr (sizeof(R) == 4) {
    /* FP32 direction: the FP64 tangent, square root and divisions are slow on
     * this GPU and the result is stored in FP32 anyway */
    const float dx = tanf((float)x1), dy = tanf((float)y1), inv = 1.0f / sqrtf(dx * dx + dy * dy + 1.0f);
    p.d[0] = dx * inv; p.d[1] = dy * inv; p.d[2] = inv;
  } else {
    double dx = tan(x1), dy = tan(y1), dz = 1.0, nn = sqrt(dx * dx + dy * dy + dz * dz);
    p.d[0] = (R)(dx / nn); p.d[1] = (R)(dy / nn); p.d[2] = (R)(dz / nn);
  }
  p.theta = acos(p.d[2]);
  p.phi = atan2(p.d[1], p.d[0]);
  bool horizontal;
  if (it.kind == 0) horizontal = xmi_rng_uniform(&g) <= hvr;
  else horizontal = (double)(it.local0 + j + 1) <= it.hor_ver_ratio;
  if (horizontal) { p.el[0] = (R)0; p.el[1] = (R)1; p.el[2] = (R)0; }
  else { p.el[0] = (R)1; p.el[1] = (R)0; p.el[2] = (R)0; }
  p.we = p.w;
  R cosalfa = rdot(p.el, p.d);
  if (fabs(cosalfa) > (R)1) return false;
  R c_alfa = acos(cosalfa);
  R c_ae = (R)1.0 / sin(c_alfa), c_be = -c_ae * cosalfa;
#pragma unroll
  for (int k = 0; k < 3; k++) p.el[k] = c_ae * p.el[k] + c_be * p.d[k];
  /* xmi_photon_shift_first_layer */
  p.layer = -1;
  if (p.c[2] >= b.zbeg[0]) {
    for (int i = 0; i < b.n_layers; i++)
      if (p.c[2] < b.zend[i]) { p.layer = i; break; }
    if (p.layer < 0) return false;
  } else {
    double ip[3], dd;
    if (!plane_step(p.c, p.d, b.n_sample, b.zbeg[0], ip, sizeof(R) == 4 ? nullptr : &dd)) return false;
    p.c[0] = ip[0]; p.c[1] = ip[1]; p.c[2] = ip[2];
    p.layer = 0;
  }
  return true;
}

/* tallies of a finished history: an analog detector hit goes to the
 * brute-force histories (and, without variance reduction, the spectrum) */
template <typename R>
__device__ __forceinline__ void finish_photon(const DevBundle<R> &b, const DevTally &t, const Photon<R> &p) {
  if (!p.hit) return;
  if (b.use_vr == 0) tally_channel(b, t, p.n_int, p.E, (double)p.w);
  if (p.n_int > 0) {
    int slot = -1;
    if (p.h_type < 0) slot = p.h_slot;
    else if (p.h_type == XMI_RAYLEIGH) slot = b.n_lines + 2 * p.h_elem;
    else if (p.h_type == XMI_COMPTON) slot = b.n_lines + 2 * p.h_elem + 1;
    if (slot >= 0 && XMI_CHK((long long)(p.n_int - 1) * b.n_slots + slot, (long long)b.N * b.n_slots, 32))
      atomicAdd(&t.hist_brute[(size_t)(p.n_int - 1) * b.n_slots + slot], (double)p.w);
  }
}

/* photon of work index w (within its configuration) at the source: false if
 * there is none (skipped draw or a source error, which is flagged) */
template <typename R>
__device__ __forceinline__ bool init_photon(const DevBundle<R> &b, const DevTally &t, long long w, Photon<R> &p) {
  int lo = 0, hi = b.n_items - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (w >= XMI_LDG(b.item_first, mid, b.n_items, 21)) lo = mid; else hi = mid - 1;
  }
  if (!XMI_CHK(lo, b.n_items, 40)) return false;
  const xmi_source_item &it = b.items[lo];
  const long long j = w - XMI_LDG(b.item_first, lo, b.n_items, 21);
  p.id = it.first + j;
  p.n_int = 0;
  p.last = XMI_NO_INTERACTION;
  p.hit = 0;
  p.h_type = XMI_NO_INTERACTION;
  p.h_elem = 0;
  p.h_slot = 0;
  p.elem = 0;
  bool skip;
  bool ok;
  if constexpr (sizeof(R) == 4) ok = start_photon_f32(b, it, j, p, skip);
  else ok = start_photon(b, it, j, p, skip);
  if (!ok) { set_error(t, kErrSource); return false; }
  return !skip;
}

}  // namespace xmi
#endif
