/*
 * Point-detector estimator kernel (src/xmi_variance_reduction.F90:29-726,
 * the element and line loops 300-709, and xmi_compton_varred2 949-1101).
 *
 * Input: the VrEvents of a chunk of photons, in an order sorted by
 * (layer, interaction order).  One lane evaluates one event; the 32 events of
 * a warp then share the layer and the order almost always, so every lane
 * walks the same element list and the same line list in lockstep: table
 * loads of a line are warp-uniform (one transaction, broadcast), nothing
 * diverges except the Compton rejection loop, and the 32 contributions to a
 * history slot are summed across the warp before one shared-memory FP64 add.
 * Warps whose events mix keys (at most one per key boundary) run the same
 * code per lane with per-lane atomics.
 *
 * Per (event, line): 8 FMA for the escape path, one exp, a handful of
 * multiplies; per (event, element): two form-factor lookups, one Doppler
 * Compton energy, one mu(E') over the layers, 9 shell probabilities.
 */
#ifndef XMIMSIM_GB300_ESTIMATOR_CUH
#define XMIMSIM_GB300_ESTIMATOR_CUH

#include "transport.cuh"

namespace xmi {

/* exp(-sum_j mu_j rho_j d_j) of a line from the sum over its line-table mu
 * (ent_pmu): the FP32 tables hold -log2(e) mu, so that the attenuation is
 * one exp2; the FP64 tables hold mu */
template <typename R>
__device__ __forceinline__ R line_atten(R s) {
  if constexpr (sizeof(R) == 4) return exp2f(s);
  else return exp(-s);
}

/* the 9 shell factors of element e at the energy of line `slot` (an event
 * of a fluorescence photon): one record of the device's precalc_xrf */
template <typename R>
__device__ __forceinline__ void xrf_at_line(const DevBundle<R> &b, int e, int slot, R *P) {
  const long long base = ((long long)e * b.n_lines + slot) * kXrfRec;
#ifndef XMI_CHECKED
  if constexpr (sizeof(R) == 4 && XMI_NSHELL == 9) {
    const float4 *p = reinterpret_cast<const float4 *>(b.precalc_xrf + base);
    const float4 a = __ldg(p), c = __ldg(p + 1), d = __ldg(p + 2);
    P[0] = a.x, P[1] = a.y, P[2] = a.z, P[3] = a.w, P[4] = c.x, P[5] = c.y, P[6] = c.z, P[7] = c.w, P[8] = d.x;
    return;
  }
#endif
#pragma unroll
  for (int s = 0; s < XMI_NSHELL; s++)
    P[s] = XMI_LDG(b.precalc_xrf, base + s, (long long)b.n_elem * b.n_lines * kXrfRec, 10);
}

/* sum_j mu_j(E) rd_j over the layers: FP32 reads the first four layers' mu
 * only when the configuration has no more (the others' mu and path sums are
 * zero) */
template <typename R>
__device__ __forceinline__ R mu_path(const DevBundle<R> &b, R E, const R *rd) {
#ifndef XMI_CHECKED
  if constexpr (sizeof(R) == 4 && XMI_MAXL == 8) {
    int node;
    float f;
    locate(b, E, node, f);
    const float4 *p = reinterpret_cast<const float4 *>(b.mu_tab + (long long)node * XMI_MAXL);
    const float4 a0 = __ldg(p), c0 = __ldg(p + 2);
    float s = (a0.x + f * (c0.x - a0.x)) * rd[0];
    s += (a0.y + f * (c0.y - a0.y)) * rd[1];
    s += (a0.z + f * (c0.z - a0.z)) * rd[2];
    s += (a0.w + f * (c0.w - a0.w)) * rd[3];
    if (b.n_layers > 4) {
      const float4 a1 = __ldg(p + 1), c1 = __ldg(p + 3);
      s += (a1.x + f * (c1.x - a1.x)) * rd[4];
      s += (a1.y + f * (c1.y - a1.y)) * rd[5];
      s += (a1.z + f * (c1.z - a1.z)) * rd[6];
      s += (a1.w + f * (c1.w - a1.w)) * rd[7];
    }
    return s;
  }
#endif
  R mus[XMI_MAXL];
  mu_calc(b, E, mus);
  R s = (R)0;
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++) s += mus[j] * rd[j];
  return s;
}

/* exp(-x) of an attenuation exponent: FP32 as exp2(-log2(e) x) */
template <typename R>
__device__ __forceinline__ R atten(R x) {
  if constexpr (sizeof(R) == 4) return exp2f(-1.44269504088896341f * x);
  else return exp(-x);
}


template <typename R>
__device__ __forceinline__ R warp_sum_r(R v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

template <typename R>
__device__ __forceinline__ void chan_add(const DevBundle<R> &b, const DevTally &t, int n, R E, R w) {
  if (w == (R)0 || E < (R)kEnergyThreshold) return;
  const int ch = channel_of(b, E);
  if (ch >= 0 && ch <= b.nch - 1 && XMI_CHK((long long)n * b.nch + ch, (long long)(b.N + 1) * b.nch, 30))
    atomicAdd(&t.chan[(size_t)n * b.nch + ch], (double)w);
}

template <typename R>
__device__ __forceinline__ void chan_add_warp(const DevBundle<R> &b, const DevTally &t, int n, R E, R w, R *buf);

/* xmi_compton_varred (src/xmi_variance_reduction.F90:752-947), the estimator
 * of the advanced Compton scattering: one scattered energy per shell of
 * element e, drawn from g for every shell with a non-zero share, each
 * weighted by that share; the spectrum gets every shell's energy.  Returns
 * the element's Compton history weight (the sum over shells).  base = the
 * event's pconv x pdir x weight (0 for an idle lane).  ch_buf: the warp's
 * channel buffer when all 32 lanes run the same element (their channel
 * contributions are then grouped by channel), nullptr for per-lane atomics. */
template <typename R>
__device__ __noinline__ R compton_advanced_est(const DevBundle<R> &b, const DevTally &t, int e, const VrEvent<R> &ev,
                                               R base, xmi_rng *g, bool valid, bool &ok, R *ch_buf) {
  using T = cp_real<R>;
  T cdfs[XMI_CP_SH];
  const T E = (T)ev.E, th = (T)ev.theta, c = cos(th), sn = sin(th), sh = sin(th * (T)0.5);
  const T sum = cp_shell_cdfs<T>(b, e, E, c, sh * sh, cdfs);
  R total = (R)0;
  const bool none = sum == (T)0;
  if (none && !ch_buf) return total;
  const int ns = b.cp_nshell[e];
  for (int k = 0; k < ns; k++) {
    R tw = (R)0;
    T ec = (T)0;
    const T sw = none ? (T)0 : (T)b.cp_occ[e * XMI_CP_SH + k] * cdfs[k] / sum;
    if (sw != (T)0) {
      const T q = cp_shell_q<T>(b.cp_qinv[e] + (size_t)k * XMI_CP_N, (T)uni<R>(g) * cdfs[k]);
      bool bad = false;
      ec = cp_energy_from_q(E, q, c, sn, bad);
      if (bad) {
        if (valid) ok = false;
        ec = (T)0;
      } else if (ec != (T)0) {
        R mus_c[XMI_MAXL];
        mu_calc(b, (R)ec, mus_c);
        R murhod = (R)0;
#pragma unroll
        for (int j = 0; j < XMI_MAXL; j++) murhod += mus_c[j] * ev.rd[j];
        tw = base * atten<R>(murhod) * (R)sw;
        total += tw;
      }
    }
    if (ch_buf) chan_add_warp(b, t, ev.n, (R)ec, valid ? tw : (R)0, ch_buf);
    else if (valid) chan_add(b, t, ev.n, (R)ec, tw);
  }
  return total;
}

/* Channel contributions of the 32 lanes of a warp (every lane calls; w = 0
 * for a lane without one): the events of a warp share configuration, layer
 * and order, and their Compton and Rayleigh energies often fall in the same
 * channel (every first-order Rayleigh contribution of a discrete line does),
 * where 32 FP64 atomics to one address serialise.  Lanes are grouped by
 * channel (match_any), the group's leader sums its peers' values from the
 * warp's buffer buf[32] in shared memory and adds the sum with one atomic. */
template <typename R>
__device__ __forceinline__ void chan_add_warp(const DevBundle<R> &b, const DevTally &t, int n, R E, R w, R *buf) {
  const int lane = threadIdx.x & 31;
  int ch = -1;
  if (w != (R)0 && E >= (R)kEnergyThreshold) {
    ch = channel_of(b, E);
    if (!(ch >= 0 && ch <= b.nch - 1 && XMI_CHK((long long)n * b.nch + ch, (long long)(b.N + 1) * b.nch, 30))) ch = -1;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, ch);
  buf[lane] = w;
  __syncwarp();
  if (ch >= 0 && lane == __ffs(peers) - 1) {
    R sum = (R)0;
    for (unsigned m = peers; m; m &= m - 1) sum += buf[__ffs(m) - 1];
    atomicAdd(&t.chan[(size_t)n * b.nch + ch], (double)sum);
  }
  __syncwarp();
}

/* History contributions of the events of one key (configuration, layer,
 * order) are summed across the warp and staged in a warp-private
 * shared-memory row, stage[j]: j < n_line = the layer's line entries (entry
 * k at j = k - first entry of the layer), then 2 i / 2 i + 1 = Rayleigh /
 * Compton of the layer's i-th element.  The row is flushed to the FP64
 * history table (one atomic per non-zero slot) when the warp's key changes. */
template <typename R>
struct StageRow {
  R *v;
  int key = -1, layer = 0, n = 1, k_first = 0, n_line = 0, size = 0;
};

template <typename R>
__device__ __forceinline__ void stage_open(const DevBundle<R> &b, StageRow<R> &st, int key, int layer, int n) {
  const int off = b.off[layer], nel = b.nel[layer];
  st.key = key;
  st.layer = layer;
  st.n = n;
  st.k_first = XMI_LDG(b.ent_off, off, b.n_layer_el + 1, 15);
  st.n_line = XMI_LDG(b.ent_off, off + nel, b.n_layer_el + 1, 15) - st.k_first;
  st.size = st.n_line + 2 * nel;
}

template <typename R>
__device__ __forceinline__ void stage_flush(const DevBundle<R> &b, const DevTally &t, StageRow<R> &st) {
  __syncwarp();
  if (st.key >= 0) {
    const long long hbase = (long long)(st.n - 1) * b.n_slots;
    const int off = b.off[st.layer];
    for (int j = threadIdx.x & 31; j < st.size; j += 32) {
      const R v = st.v[j];
      if (v == (R)0) continue;
      st.v[j] = (R)0;
      int slot;
      if (j < st.n_line) {
        slot = XMI_LDG(b.ent_slot, st.k_first + j, b.n_ent, 16);
      } else {
        const int q = j - st.n_line;
        slot = b.n_lines + 2 * XMI_LDG(b.layer_el, off + q / 2, b.n_layer_el, 9) + (q & 1);
      }
      if (XMI_CHK(hbase + slot, (long long)b.N * b.n_slots, 31)) atomicAdd(&t.hist_vr[hbase + slot], (double)v);
    }
  }
  __syncwarp();
  st.key = -1;
}

/* one contribution per lane to stage position j (Uniform: the same j in every
 * lane, warp-summed into the stage) or history slot `slot` (per-lane atomic) */
template <typename R, bool Uniform>
__device__ __forceinline__ void contribute(const DevTally &t, const StageRow<R> &st, int j, long long slot, R v) {
  if (Uniform) {
    if (__any_sync(0xffffffffu, v != (R)0)) {
      const R s = warp_sum_r(v);
      if ((threadIdx.x & 31) == 0) st.v[j] += s;
    }
  } else if (v != (R)0) {
    atomicAdd(&t.hist_vr[slot], (double)v);
  }
}

template <typename R, bool Uniform, bool Adv>
__device__ __forceinline__ void estimate_event(const DevBundle<R> &b, const DevTally &t, const StageRow<R> &st, const VrEvent<R> &ev,
                               bool valid, bool &ok) {
  const int layer = ev.layer, n = ev.n;
  const int nel = b.nel[layer], off = b.off[layer];
  const long long hbase = (long long)(n - 1) * b.n_slots;
  const int k_first = XMI_LDG(b.ent_off, off, b.n_layer_el + 1, 15);
  const int n_line = XMI_LDG(b.ent_off, off + nel, b.n_layer_el + 1, 15) - k_first;
  const R live = valid ? (R)1 : (R)0;
  R rayl_sum = (R)0; /* Rayleigh keeps the photon energy: one channel add per event */
  const ComptonEvent<R> ce = compton_event(ev.E, ev.theta);
  for (int i = 0; i < nel; i++) {
    const int pair = off + i;
    const int e = XMI_LDG(b.layer_el, pair, b.n_layer_el, 9);
    const R wi = XMI_LDG(b.layer_w, pair, b.n_layer_el, 9);
    const R pconv = wi / ev.mu_here;
    const int rs = b.n_lines + 2 * e;
    /* Rayleigh */
    const R twr = live * (pconv * (ev.pR * qtab(b.ff2[e], ev.q)) * ev.pesc_rayl * ev.w);
    contribute<R, Uniform>(t, st, n_line + 2 * i, hbase + rs, twr);
    rayl_sum += twr;
    /* Compton: one Doppler-broadened energy per element (N_COMPTON_VARRED = 1),
     * or one per shell with the advanced Compton scattering */
    xmi_rng g;
    xmi_rng_init(&g, b.seed, (uint64_t)ev.id, vr_stream(n, i));
    if (Adv && b.use_adv_compton) {
      const R twa = compton_advanced_est(b, t, e, ev, live * (pconv * (ev.pC * qtab(b.sf[e], ev.q))) * ev.w, &g,
                                         valid, ok, (R *)nullptr);
      contribute<R, Uniform>(t, st, n_line + 2 * i + 1, hbase + rs + 1, twa);
    } else {
      bool cok = true;
      const R ec = compton_energy_est(b, e, ce, &g, cok);
      R twc = (R)0;
      if (cok) {
        R mus_c[XMI_MAXL];
        mu_calc(b, ec, mus_c);
        R murhod = (R)0;
#pragma unroll
        for (int j = 0; j < XMI_MAXL; j++) murhod += mus_c[j] * ev.rd[j];
        twc = live * (pconv * (ev.pC * qtab(b.sf[e], ev.q)) * atten<R>(murhod) * ev.w);
      } else if (valid) {
        ok = false;
      }
      contribute<R, Uniform>(t, st, n_line + 2 * i + 1, hbase + rs + 1, twc);
      if (valid) chan_add(b, t, n, ec, twc);
    }
    /* fluorescence: shell probabilities at the photon energy (first order or
     * after scattering) or at the exciting line's energy (after fluorescence) */
    R P[XMI_NSHELL];
    if (ev.h_slot >= 0) {
      xrf_at_line(b, e, ev.h_slot, P);
    } else {
#pragma unroll
      for (int s = 0; s < XMI_NSHELL; s++) P[s] = el_val(b, e, XMI_REC_XRF + s, ev.node, ev.f);
    }
    if (!b.use_M_lines) {
#pragma unroll
      for (int s = 4; s < XMI_NSHELL; s++) P[s] = (R)0;
    }
    const R scale = live * wi / ev.mu_here * ev.pdir_fluo * ev.w;
    const int k0 = XMI_LDG(b.ent_off, pair, b.n_layer_el + 1, 15), k1 = XMI_LDG(b.ent_off, pair + 1, b.n_layer_el + 1, 15);
    for (int k = k0; k < k1; k++) {
      const int sl = XMI_LDG(b.ent_slot, k, b.n_ent, 16), sh = XMI_LDG(b.ent_shell, k, b.n_ent, 16);
      R ps = (R)0;
#pragma unroll
      for (int s = 0; s < XMI_NSHELL; s++)
        if (s == sh) ps = P[s];
      R murhod = (R)0;
#pragma unroll
      for (int j = 0; j < XMI_MAXL; j++)
        murhod += XMI_LDG(b.ent_pmu, (long long)k * XMI_MAXL + j, (long long)b.n_ent * XMI_MAXL, 17) * ev.rd[j];
      const R tw = ps * XMI_LDG(b.ent_coef, k, b.n_ent, 16) * scale * line_atten<R>(murhod);
      contribute<R, Uniform>(t, st, k - k_first, hbase + sl, tw);
    }
  }
  if (valid) chan_add(b, t, n, ev.E, rayl_sum);
}

/* per-warp scratch of the uniform path: the 32 events' path sums rho*d per
 * layer and, per element, shell probability x event scale */
constexpr int kScratchPerWarp = 32 * XMI_MAXL + 32 * XMI_NSHELL + 32;

/* One line entry k over the events q0 .. q0 + np2 - 1 of the warp (lane
 * group): sum of shell factor x exp(-sum_j mu_j(line) rho_j d_j).  Only the
 * first L layers are summed: the warp's configuration has at most L layers,
 * and the path sums and line mu of the others are zero, so the result is
 * the same bit for bit while the FP32 engine reads the path sums of an event
 * from shared memory in 16-byte words and does L instead of XMI_MAXL
 * multiply-adds per line and event. */
template <typename R, int L>
__device__ __forceinline__ R line_entry_events(const DevBundle<R> &b, const R *s_rd, const R *s_a, int k, int q0,
                                               int np2) {
  const int sh = XMI_LDG(b.ent_shell, k, b.n_ent, 16);
  R pmu[L];
#ifndef XMI_CHECKED
  if constexpr (sizeof(R) == 4 && XMI_MAXL == 8 && L >= 4) {
    const float4 *pp = reinterpret_cast<const float4 *>(b.ent_pmu + (long long)k * XMI_MAXL);
#pragma unroll
    for (int j4 = 0; j4 < L / 4; j4++) {
      const float4 a = __ldg(pp + j4);
      pmu[4 * j4] = a.x, pmu[4 * j4 + 1] = a.y, pmu[4 * j4 + 2] = a.z, pmu[4 * j4 + 3] = a.w;
    }
  } else if constexpr (sizeof(R) == 4 && XMI_MAXL == 8 && L == 2) {
    const float2 a = __ldg(reinterpret_cast<const float2 *>(b.ent_pmu + (long long)k * XMI_MAXL));
    pmu[0] = a.x, pmu[1] = a.y;
  } else
#endif
  {
#pragma unroll
    for (int j = 0; j < L; j++)
      pmu[j] = XMI_LDG(b.ent_pmu, (long long)k * XMI_MAXL + j, (long long)b.n_ent * XMI_MAXL, 17);
  }
  R acc = (R)0;
#pragma unroll 4
  for (int q = q0; q < q0 + np2; q++) {
    R murhod = (R)0;
    if constexpr (sizeof(R) == 4 && L >= 4) {
      const float4 *r4 = reinterpret_cast<const float4 *>(s_rd + q * XMI_MAXL);
#pragma unroll
      for (int j4 = 0; j4 < L / 4; j4++) {
        const float4 v = r4[j4];
        murhod += pmu[4 * j4] * v.x;
        murhod += pmu[4 * j4 + 1] * v.y;
        murhod += pmu[4 * j4 + 2] * v.z;
        murhod += pmu[4 * j4 + 3] * v.w;
      }
    } else if constexpr (sizeof(R) == 4 && L == 2) {
      const float2 v = *reinterpret_cast<const float2 *>(s_rd + q * XMI_MAXL);
      murhod += pmu[0] * v.x;
      murhod += pmu[1] * v.y;
    } else {
#pragma unroll
      for (int j = 0; j < L; j++) murhod += pmu[j] * s_rd[q * XMI_MAXL + j];
    }
    acc += s_a[q * XMI_NSHELL + sh] * line_atten<R>(murhod);
  }
  return acc;
}

/* The estimator for the 32 events of a warp that share configuration, layer
 * and order.  Elements: lane = event, as in the per-lane path, contributions
 * summed across the warp into the stage row.  Lines: lane = line entry, each
 * lane looping over the 32 events (their path sums and shell factors read
 * from shared memory, broadcast) and accumulating its own line's history in a
 * register -- no cross-lane reduction per line. */
template <typename R, bool Adv>
__device__ __forceinline__ void estimate_event_uniform(const DevBundle<R> &b, const DevTally &t, const StageRow<R> &st, R *scratch,
                                       const VrEvent<R> &ev, bool valid, bool &ok) {
  const int lane = threadIdx.x & 31;
  const int layer = ev.layer, n = ev.n;
  const int nel = b.nel[layer], off = b.off[layer];
  const long long hbase = (long long)(n - 1) * b.n_slots;
  R *s_rd = scratch, *s_a = scratch + 32 * XMI_MAXL, *s_ch = s_a + 32 * XMI_NSHELL;
  const R live = valid ? (R)1 : (R)0;
  R rayl_sum = (R)0; /* Rayleigh keeps the photon energy: one channel add per event */
  const ComptonEvent<R> ce = compton_event(ev.E, ev.theta);
  /* FP32: one reciprocal per event instead of a division per element */
  const R inv_mu = (R)1 / ev.mu_here;
#pragma unroll
  for (int j = 0; j < XMI_MAXL; j++) s_rd[lane * XMI_MAXL + j] = ev.rd[j];
  for (int i = 0; i < nel; i++) {
    const int pair = off + i;
    const int e = XMI_LDG(b.layer_el, pair, b.n_layer_el, 9);
    const R wi = XMI_LDG(b.layer_w, pair, b.n_layer_el, 9);
    const R pconv = sizeof(R) == 4 ? wi * inv_mu : wi / ev.mu_here;
    const int rs = b.n_lines + 2 * e;
    /* Rayleigh */
    const R twr = live * (pconv * (ev.pR * qtab(b.ff2[e], ev.q)) * ev.pesc_rayl * ev.w);
    contribute<R, true>(t, st, st.n_line + 2 * i, hbase + rs, twr);
    rayl_sum += twr;
    /* Compton: one Doppler-broadened energy per element (N_COMPTON_VARRED = 1),
     * or one per shell with the advanced Compton scattering */
    xmi_rng g;
    xmi_rng_init(&g, b.seed, (uint64_t)ev.id, vr_stream(n, i));
    if (Adv && b.use_adv_compton) {
      const R twa = compton_advanced_est(b, t, e, ev, live * (pconv * (ev.pC * qtab(b.sf[e], ev.q))) * ev.w, &g,
                                         valid, ok, s_ch);
      contribute<R, true>(t, st, st.n_line + 2 * i + 1, hbase + rs + 1, twa);
    } else {
      bool cok = true;
      const R ec = compton_energy_est(b, e, ce, &g, cok);
      R twc = (R)0;
      if (cok) {
        const R murhod = mu_path(b, ec, ev.rd);
        twc = live * (pconv * (ev.pC * qtab(b.sf[e], ev.q)) * atten<R>(murhod) * ev.w);
      } else if (valid) {
        ok = false;
      }
      contribute<R, true>(t, st, st.n_line + 2 * i + 1, hbase + rs + 1, twc);
      chan_add_warp(b, t, n, ec, valid ? twc : (R)0, s_ch);
    }
    /* shell factors of this event for element i */
    R P[XMI_NSHELL];
    if (ev.h_slot >= 0) {
      xrf_at_line(b, e, ev.h_slot, P);
    } else {
      el_xrf(b, e, ev.node, ev.f, P);
    }
    const R scale = live * (sizeof(R) == 4 ? wi * inv_mu : wi / ev.mu_here) * ev.pdir_fluo * ev.w;
#pragma unroll
    for (int s = 0; s < XMI_NSHELL; s++)
      s_a[lane * XMI_NSHELL + s] = (s >= 4 && !b.use_M_lines) ? (R)0 : P[s] * scale;
    __syncwarp();
    /* lines of element i: with nl entries, np2 = the smallest power of two
     * >= nl (at most 32) lanes take one entry each and the 32 / np2 groups of
     * lanes split the warp's events (np2 each), their partial sums combined by
     * shuffles -- an element with few lines still keeps the warp busy */
    const int k0 = XMI_LDG(b.ent_off, pair, b.n_layer_el + 1, 15), k1 = XMI_LDG(b.ent_off, pair + 1, b.n_layer_el + 1, 15);
    int np2 = 1;
    while (np2 < k1 - k0 && np2 < 32) np2 <<= 1;
    const int li = lane & (np2 - 1), q0 = lane - li; /* q0 = group x np2: the group's first event */
    const int nL = b.n_layers; /* warp-uniform: one configuration per warp here */
    for (int kb = k0; kb < k1; kb += np2) {
      const int k = kb + li;
      R acc = (R)0;
      if (k < k1) {
        if (XMI_MAXL == 8 && nL <= 2) acc = line_entry_events<R, (XMI_MAXL < 2 ? XMI_MAXL : 2)>(b, s_rd, s_a, k, q0, np2);
        else if (XMI_MAXL == 8 && nL <= 4) acc = line_entry_events<R, (XMI_MAXL < 4 ? XMI_MAXL : 4)>(b, s_rd, s_a, k, q0, np2);
        else acc = line_entry_events<R, XMI_MAXL>(b, s_rd, s_a, k, q0, np2);
      }
      for (int off = np2; off < 32; off <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (q0 == 0 && k < k1) st.v[k - st.k_first] += acc * XMI_LDG(b.ent_coef, k, b.n_ent, 16);
    }
    __syncwarp();
  }
  chan_add_warp(b, t, n, ev.E, valid ? rayl_sum : (R)0, s_ch);
}

/* number of events the queue holds: the count, capped at the capacity (a
 * count past the capacity means events were dropped and the run is flagged) */
__device__ __forceinline__ long long queued_events(const unsigned long long *count, long long cap) {
  const long long n = (long long)*count;
  return n < cap ? n : cap;
}

/* an event the transport kernel could not have produced is replaced by a
 * harmless one (and refused by the caller) */
template <typename R>
__device__ __forceinline__ bool event_in_range(const DevBundle<R> &b, VrEvent<R> &ev, int n_cfg) {
  if (ev.layer >= 0 && ev.layer < b.n_layers && ev.n >= 1 && ev.n <= b.N && ev.h_slot < b.n_lines && ev.cfg >= 0 &&
      ev.cfg < n_cfg)
    return true;
  ev.layer = 0;
  ev.n = 1;
  ev.h_slot = -1;
  ev.cfg = 0;
  return false;
}

/* events per work grab of a warp: consecutive in the sorted order, so a
 * warp's stage row keeps its key across grabs */
constexpr int kEventsPerGrab = 256;

/* Estimator over the events [0, min(*count, cap)) of the queue in `order`;
 * bundles[cfg] / tallies[cfg] of each event's configuration (one entry when
 * not batched).  Warps grab kEventsPerGrab consecutive events at a time from
 * the counter `work`; stage rows of stage_cap values per warp sit in dynamic
 * shared memory. */
template <typename R, bool Adv = false>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 3) estimator_kernel(const DevBundle<R> *bundles, const DevTally *tallies,
                                                           int n_cfg, const VrEvent<R> *events, const int *order,
                                                           const unsigned long long *count, long long cap,
                                                           unsigned long long *work, int stage_cap,
                                                           unsigned long long *flags) {
  extern __shared__ unsigned char stage_mem[];
  StageRow<R> st;
  st.v = (R *)stage_mem + (size_t)(threadIdx.x >> 5) * (stage_cap + kScratchPerWarp);
  R *scratch = st.v + stage_cap;
  const int lane = threadIdx.x & 31;
  for (int j = lane; j < stage_cap; j += 32) st.v[j] = (R)0;
  __syncwarp();
  int st_cfg = 0;
  const long long n_ev = queued_events(count, cap);
  bool ok = true;
  for (;;) {
    unsigned long long grab = 0;
    if (lane == 0) grab = atomicAdd(work, (unsigned long long)kEventsPerGrab);
    grab = __shfl_sync(0xffffffffu, grab, 0);
    if ((long long)grab >= n_ev) break;
    for (int sub = 0; sub < kEventsPerGrab; sub += 32) {
      const long long base = (long long)grab + sub;
      if (base >= n_ev) break;
      const long long k = base + lane;
      bool valid = k < n_ev;
      /* lanes past the end carry the warp's first event with zero weight */
      long long oi = order[valid ? k : base];
      if (oi < 0 || oi >= n_ev) { oi = 0; valid = false; ok = false; }
      VrEvent<R> ev = events[oi];
      if (ev.cfg < 0 || ev.cfg >= n_cfg) { ev.cfg = 0; valid = false; ok = false; }
      const DevBundle<R> &b = bundles[ev.cfg];
      if (!event_in_range(b, ev, n_cfg)) { valid = false; ok = false; }
      const DevTally &t = tallies[ev.cfg];
      const int key = vr_key(ev);
      if (__all_sync(0xffffffffu, key == __shfl_sync(0xffffffffu, key, 0))) {
        if (key != st.key) {
          stage_flush(bundles[st_cfg], tallies[st_cfg], st);
          if (b.stage_max <= stage_cap) {
            stage_open(b, st, key, ev.layer, ev.n);
            st_cfg = ev.cfg;
          }
        }
        if (st.key == key) estimate_event_uniform<R, Adv>(b, t, st, scratch, ev, valid, ok);
        else estimate_event<R, false, Adv>(b, t, st, ev, valid, ok);
      } else {
        estimate_event<R, false, Adv>(b, t, st, ev, valid, ok);
      }
    }
  }
  stage_flush(bundles[st_cfg], tallies[st_cfg], st);
  if (!ok) atomicCAS(flags, 0ull, kErrCompton);
}

/* counting sort of the chunk's events by key (vr_key): histogram, exclusive
 * scan, scatter.  A block takes a contiguous range of the queue, where few
 * keys occur (the queue fills round by round, photon by photon, and a chunk
 * spans a few configurations): it counts its keys in a shared-memory table
 * (one shared atomic per group of equal keys in a warp) and adds each key's
 * count to the global histogram once, instead of every warp's groups
 * contending for the same few global counters.  A key that finds the table
 * full is counted with global atomics (the probe loop is bounded by the
 * table size). */
constexpr int kSortSlots = 1024;

/* slot of `k` in a block's key table (linear probing from a multiplicative
 * hash); insert: claim an empty slot for it; -1: not found / table full */
__device__ __forceinline__ int sort_slot(volatile int *keys, int k, bool insert) {
  int s = (int)(((unsigned)k * 2654435761u) >> 22); /* top 10 bits */
  for (int probe = 0; probe < kSortSlots; probe++) {
    const int cur = keys[s];
    if (cur == k) return s;
    if (cur == -1) {
      if (!insert) return -1;
      const int old = atomicCAS((int *)&keys[s], -1, k);
      if (old == -1 || old == k) return s;
      if (keys[s] == k) return s;
    }
    s = (s + 1) & (kSortSlots - 1);
  }
  return -1;
}

/* the block's contiguous share [r0, r1) of the n queued events (a multiple of 32 long) */
__device__ __forceinline__ void sort_range(long long n, long long &r0, long long &r1) {
  const long long per = ((n + gridDim.x - 1) / gridDim.x + 31) & ~31ll;
  r0 = (long long)blockIdx.x * per;
  r1 = r0 + per < n ? r0 + per : n;
}

/* groups of equal keys in a warp: consecutive events mostly share theirs,
 * and one vote settles that case */
__device__ __forceinline__ unsigned key_peers(int k) {
  return __all_sync(0xffffffffu, k == __shfl_sync(0xffffffffu, k, 0)) ? 0xffffffffu
                                                                     : __match_any_sync(0xffffffffu, k);
}

/* counts of the block's range into the table s_key / s_cnt (keys without a
 * slot go straight to `spill`, when given) */
__device__ __forceinline__ void count_block_keys(const int *key, long long r0, long long r1, int nkeys, int *s_key,
                                                 unsigned *s_cnt, unsigned *spill) {
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (long long base = r0 + (long long)(threadIdx.x >> 5) * 32; base < r1; base += (long long)nw * 32) {
    const long long i = base + lane;
    const int k = i < r1 ? key[i] : -1;
    const unsigned peers = key_peers(k);
    if (k >= 0 && k < nkeys && lane == __ffs(peers) - 1) {
      const int sl = sort_slot(s_key, k, true);
      if (sl >= 0) atomicAdd(&s_cnt[sl], (unsigned)__popc(peers));
      else if (spill) atomicAdd(&spill[k], (unsigned)__popc(peers));
    }
  }
}

__global__ void __launch_bounds__(256) event_key_histogram(const int *key, const unsigned long long *count,
                                                           long long cap, int nkeys, unsigned *hist) {
  __shared__ int s_key[kSortSlots];
  __shared__ unsigned s_cnt[kSortSlots];
  for (int j = threadIdx.x; j < kSortSlots; j += blockDim.x) s_key[j] = -1, s_cnt[j] = 0u;
  __syncthreads();
  long long r0, r1;
  sort_range(queued_events(count, cap), r0, r1);
  count_block_keys(key, r0, r1, nkeys, s_key, s_cnt, hist);
  __syncthreads();
  for (int j = threadIdx.x; j < kSortSlots; j += blockDim.x)
    if (s_key[j] >= 0 && s_cnt[j] != 0u) atomicAdd(&hist[s_key[j]], s_cnt[j]);
}

/* exclusive scan of the key counts into the scatter cursors; also adds the
 * chunk's event count to the run total */
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) event_key_scan(const unsigned *hist, int nkeys, unsigned *cursor,
                                                               const unsigned long long *count,
                                                               unsigned long long *total) {
  /* one block: each thread scans a contiguous run of keys; the runs' sums
   * are scanned across the block */
  __shared__ unsigned part[kScanThreads];
  const int per = (nkeys + kScanThreads - 1) / kScanThreads;
  const int k0 = threadIdx.x * per, k1 = k0 + per < nkeys ? k0 + per : nkeys;
  unsigned sum = 0;
  for (int k = k0; k < k1; k++) sum += hist[k];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int d = 1; d < kScanThreads; d <<= 1) {
    const unsigned v = threadIdx.x >= d ? part[threadIdx.x - d] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned acc = part[threadIdx.x] - sum;
  for (int k = k0; k < k1; k++) {
    cursor[k] = acc;
    acc += hist[k];
  }
  if (threadIdx.x == 0) *total += *count;
}

/* positions: the block counts its range's keys again, reserves one run of
 * positions per key with one global atomic, then hands out positions within
 * each run with shared atomics (keys without a slot take theirs from the
 * global cursor per warp group) */
__global__ void __launch_bounds__(256) event_key_scatter(const int *key, const unsigned long long *count,
                                                         long long cap, int nkeys, unsigned *cursor, int *order) {
  __shared__ int s_key[kSortSlots];
  __shared__ unsigned s_cnt[kSortSlots], s_base[kSortSlots];
  for (int j = threadIdx.x; j < kSortSlots; j += blockDim.x) s_key[j] = -1, s_cnt[j] = 0u;
  __syncthreads();
  const long long n = queued_events(count, cap);
  long long r0, r1;
  sort_range(n, r0, r1);
  count_block_keys(key, r0, r1, nkeys, s_key, s_cnt, nullptr);
  __syncthreads();
  for (int j = threadIdx.x; j < kSortSlots; j += blockDim.x)
    if (s_key[j] >= 0) {
      s_base[j] = s_cnt[j] != 0u ? atomicAdd(&cursor[s_key[j]], s_cnt[j]) : 0u;
      s_cnt[j] = 0u;
    }
  __syncthreads();
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (long long base = r0 + (long long)(threadIdx.x >> 5) * 32; base < r1; base += (long long)nw * 32) {
    const long long i = base + lane;
    const int k = i < r1 ? key[i] : -1;
    const unsigned peers = key_peers(k);
    if (k >= 0 && k < nkeys) {
      const int leader = __ffs(peers) - 1;
      unsigned pos = 0;
      if (lane == leader) {
        const int sl = sort_slot(s_key, k, false);
        pos = sl >= 0 ? s_base[sl] + atomicAdd(&s_cnt[sl], (unsigned)__popc(peers))
                      : atomicAdd(&cursor[k], (unsigned)__popc(peers));
      }
      pos = __shfl_sync(peers, pos, leader) + __popc(peers & ((1u << lane) - 1u));
      if ((long long)pos < n) order[pos] = (int)i;
    }
  }
}

}  // namespace xmi
#endif
