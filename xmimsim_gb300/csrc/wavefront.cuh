/*
 * Wavefront (event-based) transport: the photons of a chunk advance one step
 * at a time through small kernels, re-queued per interaction type with
 * warp-aggregated appends, instead of one thread following one history
 * through every code path.
 *
 *   wf_start     source sampling of the chunk's work indices   -> active list
 *   wf_step      transport to the next interaction, estimator event, atom and
 *                interaction type (step_photon)                 -> Rayleigh /
 *                                                                  Compton /
 *                                                                  photo queue
 *   wf_interact  one interaction type per launch (interact)    -> next active
 *
 * A photon's draws are those of the history kernel: the step kernel saves the
 * position in the step's Philox stream and the interaction kernel resumes it.
 * Each kernel runs one code path for all its lanes, so warps stay converged
 * and the instruction working set stays small.
 */
#ifndef XMIMSIM_GB300_WAVEFRONT_CUH
#define XMIMSIM_GB300_WAVEFRONT_CUH

#include "transport.cuh"

namespace xmi {

/* photon state between wavefront kernels */
template <typename R>
struct __align__(16) WfPhoton {
  Photon<R> p;
  uint32_t ctr0; /* next block of the step's Philox stream */
  int pos;       /* draws taken from the block before it (2: none left) */
  int cfg;       /* configuration of a batched run */
};

/* lists of one chunk: two active lists (alternating), three interaction queues */
struct WfLists {
  int *active[2];
  int *inter[3];   /* Rayleigh, Compton, photoelectric */
  unsigned *count; /* [0], [1] active lists, [2..4] interaction queues */
  /* analog cascades: the photons of the chunk sit in slots [0, half), the
   * offspring of slot i in slot half + i; casc[i] != 0 once photon i's
   * cascade has happened */
  unsigned char *casc;
  long long half;
};

/* appends `value` to `list`; lanes appending to the same list share one atomic */
__device__ __forceinline__ void wf_append(int *list, unsigned *count, int value) {
  const unsigned mask = __activemask();
  const unsigned peers = __match_any_sync(mask, (unsigned long long)(size_t)count);
  const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(count, (unsigned)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  list[base + __popc(peers & ((1u << lane) - 1u))] = value;
}

template <typename R, bool Batched>
__device__ __forceinline__ const DevBundle<R> &wf_bundle(const DevBundle<R> &b0, const DevBundle<R> *bundles, int c) {
  return Batched ? bundles[c] : b0;
}
template <bool Batched>
__device__ __forceinline__ const DevTally &wf_tally(const DevTally &t0, const DevTally *tallies, int c) {
  return Batched ? tallies[c] : t0;
}

/* work indices [w0, w1) of the configuration(s): cfg_first[c] = first work
 * index of configuration c (n_cfg + 1 entries) when batched */
template <typename R, bool Batched>
__global__ void __launch_bounds__(128) wf_start(DevBundle<R> b0, DevTally t0, const DevBundle<R> *bundles,
                                                const DevTally *tallies, const long long *cfg_first, int n_cfg,
                                                long long w0, long long w1, WfPhoton<R> *st, WfLists q) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long w = w0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; w < w1; w += stride) {
    int c = 0;
    long long wl = w;
    if (Batched) {
      /* the warp's work indices are consecutive: the first active lane finds
       * its configuration by bisection and every lane steps forward from it
       * (a warp spans few configurations) */
      const unsigned act = __activemask();
      const int lead = __ffs(act) - 1;
      int lo = 0;
      if ((int)(threadIdx.x & 31) == lead) {
        int hi = n_cfg - 1;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (w >= __ldg(cfg_first + mid)) lo = mid; else hi = mid - 1;
        }
      }
      lo = __shfl_sync(act, lo, lead);
      while (lo + 1 < n_cfg && w >= __ldg(cfg_first + lo + 1)) lo++;
      c = lo;
      wl = w - __ldg(cfg_first + lo);
    }
    WfPhoton<R> x;
    if (!init_photon(wf_bundle<R, Batched>(b0, bundles, c), wf_tally<Batched>(t0, tallies, c), wl, x.p)) continue;
    x.ctr0 = 0u;
    x.pos = 2;
    x.cfg = c;
    const int slot = (int)(w - w0);
    st[slot] = x;
    wf_append(q.active[0], &q.count[0], slot);
  }
}

/* clears the lists the next iteration fills */
__global__ void wf_reset(WfLists q, int next) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    q.count[next] = 0u;
    q.count[2] = q.count[3] = q.count[4] = 0u;
  }
}

/* FP32: at most 128 registers, four blocks of 128 per SM (the unbounded
 * build takes 146 registers and fits three; bounded it spills 12 bytes);
 * FP64: three blocks, as unbounded */
template <typename R, bool Batched>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 4 : 3) wf_step(DevBundle<R> b0, DevTally t0, const DevBundle<R> *bundles,
                                               const DevTally *tallies, WfPhoton<R> *st, WfLists q, int cur,
                                               long long cap, VrQueue<R> vq) {
  const long long n = (long long)q.count[cur] < cap ? (long long)q.count[cur] : cap;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int slot = q.active[cur][i];
    if (slot < 0 || slot >= cap) continue;
    WfPhoton<R> x = st[slot];
    const DevBundle<R> &b = wf_bundle<R, Batched>(b0, bundles, x.cfg);
    const DevTally &t = wf_tally<Batched>(t0, tallies, x.cfg);
    xmi_rng g;
    const int s = step_photon(b, x.p, t, vq, x.cfg, g);
    if (s == kStepDone) {
      finish_photon(b, t, x.p);
      continue;
    }
    if (s != kStepInteract) continue;
    x.ctr0 = g.ctr.v[0];
    x.pos = g.pos;
    st[slot] = x;
    const int k = x.p.last == XMI_RAYLEIGH ? 0 : (x.p.last == XMI_COMPTON ? 1 : 2);
    wf_append(q.inter[k], &q.count[2 + k], slot);
  }
}

/* the photons of interaction queue k (0 Rayleigh, 1 Compton, 2 photoelectric);
 * Adv: with the advanced Compton scattering compiled in; Casc (queue 2 only):
 * with the analog cascades, which start offspring photons in slots
 * [half, 2 half) */
template <typename R, bool Batched, bool Adv = false, bool Casc = false>
__global__ void __launch_bounds__(128) wf_interact(DevBundle<R> b0, DevTally t0, const DevBundle<R> *bundles,
                                                   const DevTally *tallies, WfPhoton<R> *st, WfLists q, int k,
                                                   int next, long long cap) {
  const long long n = (long long)q.count[2 + k] < cap ? (long long)q.count[2 + k] : cap;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int slot = q.inter[k][i];
    if (slot < 0 || slot >= cap) continue;
    WfPhoton<R> x = st[slot];
    const DevBundle<R> &b = wf_bundle<R, Batched>(b0, bundles, x.cfg);
    const DevTally &t = wf_tally<Batched>(t0, tallies, x.cfg);
    xmi_rng g;
    xmi_rng_resume(&g, b.seed, (uint64_t)x.p.id, (uint32_t)x.p.n_int, x.ctr0, x.pos);
    if constexpr (Casc) {
      WfPhoton<R> y;
      int flags = slot < q.half && slot + q.half < cap && q.casc[slot] == 0 ? kCascAllowed : 0;
      if (!fluorescence<R, true>(b, x.p, &g, &y.p, &flags)) {
        set_error(t, kErrTable);
        continue;
      }
      if (flags & kCascUsed) q.casc[slot] = 1;
      if (flags & kCascChild) {
        y.ctr0 = 0u;
        y.pos = 2;
        y.cfg = x.cfg;
        st[slot + q.half] = y;
        wf_append(q.active[next], &q.count[next], (int)(slot + q.half));
      }
    } else {
      if (!interact<R, Adv>(b, x.p, t, g)) continue;
    }
    st[slot] = x;
    wf_append(q.active[next], &q.count[next], slot);
  }
}

}  // namespace xmi
#endif
