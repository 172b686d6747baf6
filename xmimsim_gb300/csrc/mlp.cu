/*
 * Solid-angle surrogate network on the fifth-generation tensor cores.
 *
 * The network maps a point in the sample frame, given as three features
 * (distance to the detector centre, axial distance, cosine of the angle to
 * the detector axis), to log(solid angle):
 *     h0 = SiLU(W0 x + b0), h_l = SiLU(W_l h_{l-1} + b_l) (l = 1..3),
 *     y = w_o . h3 + b_o,
 * hidden width 128, BF16 weights and activations, FP32 accumulation.
 *
 * Parameter vector (FP32 master copy, MLP_NPARAM values):
 *     W0 [128][3], b0 [128], then for l = 1..3: W_l [128][128], b_l [128],
 *     then w_o [128], b_o.
 *
 * Layer 0 (three FP32 inputs) runs on the CUDA cores in FP32: BF16 inputs
 * would quantise the features to 2^-9 of their range, far coarser than the
 * solid angle varies.  Layers 1-3 run on the tensor cores.
 *
 * Forward kernel: one CTA of 128 threads per SM, weights resident in shared
 * memory (packed once per launch), 128 queries per tile.  Thread t owns
 * query row t of the tile: it computes the row's layer-0 activations, writes
 * them into the K-major operand tile, and after each tensor-core layer reads
 * its accumulator row back from tensor memory (TMEM lanes 32 w .. 32 w + 31
 * belong to warp w).  Thread 0 issues the MMAs, eight K16 steps per layer.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "solid_angle.cuh"
#include "umma.cuh"
#include "xmi_internal.h"

namespace xmi {
namespace mlp {

constexpr int H = 128;    /* hidden width */
constexpr int KIN = 16;   /* input features padded to one K step */
constexpr int NIN = 3;
constexpr int NPARAM = H * NIN + H + 3 * (H * H + H) + H + 1;
constexpr int OFF_W0 = 0, OFF_B0 = H * NIN;
__host__ __device__ constexpr int off_w(int l) { return OFF_B0 + H + (l - 1) * (H * H + H); }
__host__ __device__ constexpr int off_b(int l) { return off_w(l) + H * H; }
constexpr int OFF_WO = OFF_B0 + H + 3 * (H * H + H), OFF_BO = OFF_WO + H;

/* bytes of the packed BF16 weight tiles: W0 [128 x 16], W1..W3 [128 x 128] */
constexpr int W0_BYTES = H * KIN * 2, WL_BYTES = H * H * 2;
constexpr int PACK_BYTES = W0_BYTES + 3 * WL_BYTES;

/* The forward kernels run three independent groups of 128 threads per CTA,
 * each with its own 128-row tile, activation tile, TMEM accumulator and
 * mbarrier, sharing the resident weights: while one group's SiLU epilogue
 * runs on the CUDA cores another's MMAs run on the tensor cores. */
constexpr int kGroups = 3, kFwdThreads = 128 * kGroups;
constexpr uint32_t kTmemCols = 512; /* power of two >= 128 kGroups */

/* shared-memory plan of the forward kernels (offsets in bytes) */
constexpr int SM_W = 0;                           /* packed weights */
constexpr int SM_X0 = SM_W + PACK_BYTES;          /* FP32 W0 of layer 0 */
constexpr int SM_A = SM_X0 + H * KIN * 2;         /* kGroups activation tiles [128 x 128] */
constexpr int SM_BIAS = SM_A + kGroups * H * H * 2; /* b0..b3 FP32 */
constexpr int SM_WO = SM_BIAS + 4 * H * 4;        /* w_o FP32 */
constexpr int SM_BAR = SM_WO + H * 4;             /* kGroups mbarriers, TMEM address */
constexpr int SM_TOTAL = SM_BAR + 8 * kGroups + 16;
static_assert(SM_TOTAL <= 227 * 1024, "forward kernel shared memory");

/* barrier and vote among the 128 threads of one group (named barrier 1 + g) */
__device__ __forceinline__ void group_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }
__device__ __forceinline__ bool group_any(int g, bool v) {
  int r;
  asm volatile(
      "{\n"
      ".reg .pred p, q;\n"
      "setp.ne.b32 p, %1, 0;\n"
      "bar.red.or.pred q, %2, 128, p;\n"
      "selp.b32 %0, 1, 0, q;\n"
      "}\n"
      : "=r"(r)
      : "r"((int)v), "r"(1 + g)
      : "memory");
  return r != 0;
}

/* packs the FP32 weights into BF16 K-major operand tiles */
__global__ void pack_weights(const float *theta, unsigned char *packed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  /* W0: rows = output unit, K = input feature (padded with zeros) */
  if (i < H * KIN) {
    const int o = i / KIN, k = i % KIN;
    const float v = k < NIN ? theta[OFF_W0 + o * NIN + k] : 0.0f;
    *(__nv_bfloat16 *)(packed + umma::kmajor_offset(o, k, KIN)) = __float2bfloat16_rn(v);
  }
  if (i < 3 * H * H) {
    const int l = 1 + i / (H * H), r = i % (H * H), o = r / H, k = r % H;
    *(__nv_bfloat16 *)(packed + W0_BYTES + (l - 1) * WL_BYTES + umma::kmajor_offset(o, k, H)) =
        __float2bfloat16_rn(theta[off_w(l) + o * H + k]);
  }
}

/* logistic function as 1/2 + tanh(z/2)/2 with the hardware tanh
 * approximation (one MUFU op, relative error about 2^-11, below the BF16
 * rounding the activations get) -- used by inference and training alike */
__device__ __forceinline__ float sigmoid_fast(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
  return fmaf(0.5f, t, 0.5f);
}
__device__ __forceinline__ float silu(float z) { return z * sigmoid_fast(z); }
/* SiLU(z) from h = z / 2: z sigmoid(z) = z (1 + tanh(z/2)) / 2 = h + h tanh(h),
 * one MUFU op and one FMA (the inference pass gets h directly from weights
 * and biases halved in shared memory, exact in binary) */
__device__ __forceinline__ float silu_half(float h) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}

/* eight consecutive activations of one row as one 16-byte store of the
 * K-major BF16 operand tile (k0 a multiple of 8) */
__device__ __forceinline__ void store_bf16x8(unsigned char *a_tile, int row, int k0, const float *h) {
  uint4 u;
  __nv_bfloat162 p0 = __floats2bfloat162_rn(h[0], h[1]), p1 = __floats2bfloat162_rn(h[2], h[3]);
  __nv_bfloat162 p2 = __floats2bfloat162_rn(h[4], h[5]), p3 = __floats2bfloat162_rn(h[6], h[7]);
  u.x = *reinterpret_cast<uint32_t *>(&p0);
  u.y = *reinterpret_cast<uint32_t *>(&p1);
  u.z = *reinterpret_cast<uint32_t *>(&p2);
  u.w = *reinterpret_cast<uint32_t *>(&p3);
  *reinterpret_cast<uint4 *>(a_tile + umma::kmajor_offset(row, k0, H)) = u;
}

/* per-CTA context of the tensor-core forward pass (weights resident in
 * shared memory, one 128-column TMEM accumulator) */
struct FwdCtx {
  uint64_t *mbar;
  float *bias, *wo;
  unsigned char *a_tile;  /* this group's activation tile */
  float bo;
  int g, row;             /* group, tile row of this thread */
  uint32_t tmem, dcol, trow, s_a, s_w, phase;
};

__device__ void fwd_setup(unsigned char *sm, const unsigned char *packed, const float *theta, FwdCtx &c) {
  const int tid = threadIdx.x, warp = tid >> 5;
  c.g = tid >> 7;
  c.row = tid & 127;
  c.mbar = (uint64_t *)(sm + SM_BAR) + c.g;
  uint32_t *tmem_slot = (uint32_t *)(sm + SM_BAR + 8 * kGroups);
  c.bias = (float *)(sm + SM_BIAS);
  c.wo = (float *)(sm + SM_WO);
  /* every layer's weights and biases halved (W0, b0 below): the accumulators
   * then hold z / 2, the input of silu_half (a power-of-two scale: the BF16
   * weights and the FP32 accumulation round exactly as unscaled) */
  for (int i = tid; i < PACK_BYTES / 16; i += blockDim.x) {
    uint4 u = ((const uint4 *)packed)[i];
    if (i * 16 >= W0_BYTES) {
      __nv_bfloat162 *p2 = reinterpret_cast<__nv_bfloat162 *>(&u);
      const __nv_bfloat162 half2 = __float2bfloat162_rn(0.5f);
#pragma unroll
      for (int k = 0; k < 4; k++) p2[k] = __hmul2(p2[k], half2);
    }
    ((uint4 *)(sm + SM_W))[i] = u;
  }
  for (int i = tid; i < H; i += blockDim.x) {
    c.bias[i] = 0.5f * theta[OFF_B0 + i];
    for (int l = 1; l <= 3; l++) c.bias[l * H + i] = 0.5f * theta[off_b(l) + i];
    c.wo[i] = theta[OFF_WO + i];
  }
  /* FP32 W0 of the CUDA-core layer 0 (halved, as the others), in the
   * (otherwise unused) input-tile area */
  float *w0 = (float *)(sm + SM_X0);
  for (int i = tid; i < H * NIN; i += blockDim.x) w0[i] = 0.5f * theta[OFF_W0 + i];
  c.bo = theta[OFF_BO];
  if (warp == 0) umma::tmem_alloc(tmem_slot, kTmemCols);
  if (tid == 0) {
    for (int g = 0; g < kGroups; g++) umma::mbar_init((uint64_t *)(sm + SM_BAR) + g, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_proxy_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  c.tmem = *tmem_slot;
  c.dcol = c.tmem + (uint32_t)(c.g * 128);
  /* a warp reads TMEM lanes 32 (warp % 4) .. +31: its group's tile rows */
  c.trow = c.dcol + ((uint32_t)((warp & 3) * 32) << 16);
  c.a_tile = sm + SM_A + c.g * H * H * 2;
  c.s_a = umma::smem_u32(c.a_tile);
  c.s_w = umma::smem_u32(sm + SM_W);
  c.phase = 0;
}

/* layer 0 of this thread's row in FP32 on the CUDA cores (w0 and b0 halved:
 * z / 2 comes out of the FMAs); BF16 activations into the operand tile */
__device__ __forceinline__ void layer0_row(unsigned char *a_tile, int row, const float *w0, const float *b0,
                                           const float *f) {
#pragma unroll 1
  for (int j0 = 0; j0 < H; j0 += 8) {
    float h[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int j = j0 + u;
      const float zh = b0[j] + w0[j * NIN] * f[0] + w0[j * NIN + 1] * f[1] + w0[j * NIN + 2] * f[2];
      h[u] = silu_half(zh);
    }
    store_bf16x8(a_tile, row, j0, h);
  }
}

/* network output for this thread's feature row f (tile row = thread); all
 * 128 threads call it together; false (for every thread) when a wait ran out */
__device__ bool fwd_tile(unsigned char *sm, FwdCtx &c, const float *f, float &y) {
  const uint32_t idesc = umma::idesc_bf16_f32(128, 128);
  layer0_row(c.a_tile, c.row, (const float *)(sm + SM_X0), c.bias, f);
  y = c.bo;
  for (int l = 1; l < 4; l++) {
    umma::fence_proxy_async_smem();
    umma::fence_before_sync();
    group_sync(c.g);
    if (c.row == 0) {
      umma::fence_after_sync();
      const uint32_t wl = c.s_w + W0_BYTES + (l - 1) * WL_BYTES;
#pragma unroll
      for (int kk = 0; kk < H / 16; kk++)
        umma::mma_bf16(c.dcol, umma::smem_desc(c.s_a + kk * 256, 128, 2048), umma::smem_desc(wl + kk * 256, 128, 2048),
                       idesc, kk > 0);
      umma::mma_commit(c.mbar);
    }
    const bool ok = umma::mbar_wait(c.mbar, c.phase);
    c.phase ^= 1u;
    if (group_any(c.g, !ok)) return false;
    umma::fence_after_sync();
    /* epilogue of layer l: bias, SiLU (of the halved pre-activation); the
     * next layer's operand or the output */
#pragma unroll 1
    for (int q = 0; q < H / 32; q++) {
      float v[32];
      umma::tmem_ld_32x32b_x32(c.trow + q * 32, v);
#pragma unroll
      for (int j = 0; j < 32; j++) v[j] = silu_half(v[j] + c.bias[l * H + q * 32 + j]);
      if (l < 3) {
#pragma unroll
        for (int j8 = 0; j8 < 32; j8 += 8) store_bf16x8(c.a_tile, c.row, q * 32 + j8, v + j8);
      } else {
#pragma unroll
        for (int j = 0; j < 32; j++) y += v[j] * c.wo[q * 32 + j];
      }
    }
  }
  return true;
}

__device__ void fwd_teardown(FwdCtx &c) {
  umma::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) umma::tmem_dealloc(c.tmem, kTmemCols);
}

/* features [n][3] (already scaled) -> out [n] = network output (log solid
 * angle); *err set non-zero when a wait ran out */
__global__ void __launch_bounds__(kFwdThreads, 1) forward_kernel(const unsigned char *packed, const float *theta,
                                                                 const float *features, float *out, int n, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  FwdCtx c;
  fwd_setup(sm, packed, theta, c);
  bool failed = false;
  for (int tile = blockIdx.x * kGroups + c.g; tile * 128 < n; tile += gridDim.x * kGroups) {
    const int row = tile * 128 + c.row;
    const bool valid = row < n;
    float f[NIN], y;
    for (int k = 0; k < NIN; k++) f[k] = valid ? features[(size_t)row * NIN + k] : 0.0f;
    if (!fwd_tile(sm, c, f, y)) {
      failed = true;
      break;
    }
    if (valid) out[row] = y;
  }
  if (failed && c.row == 0) atomicExch(err, 1);
  fwd_teardown(c);
}

/* ---------------- surrogate of the solid-angle grid ---------------- */
/* Input scaling and checked region.  Raw features of a point (r, theta):
 * log r, the axial distance r sin(theta), and sin(theta) = cosine of the
 * angle to the detector axis; each mapped to [-1, 1] over the range the
 * training points cover.  The (log r, theta) box of the training points is
 * split into ncr x nct cells, each checked against the integrator (flag 1:
 * use the integrator there). */
struct Domain {
  float fmid[3], fhalf[3];
  float lr0, lr1, t0, t1; /* checked box */
  float tmin;             /* below the grid's lowest theta the solid angle is 0 */
  int ncr, nct;
  float eps;              /* log target = log(omega + eps) */
};

/* Flagged cells keep the integrator as their solid angle, tabulated: the
 * integrator's values on a (kPatch + 1)^2 lattice of nodes spanning the cell
 * in (log r, theta), interpolated bilinearly -- the reference grid's method
 * (integrator values at nodes, bilinear in between) at a node spacing finer
 * than its 1024 x 1024 grid over this region. */
constexpr int kPatch = 8, kPatchNodes = (kPatch + 1) * (kPatch + 1);

__host__ __device__ __forceinline__ float patch_omega(const Domain &d, const float *patch, float lr, float t, int cell) {
  const int cr = cell % d.ncr, ct = cell / d.ncr;
  const float dlr = (d.lr1 - d.lr0) / d.ncr, dt = (d.t1 - d.t0) / d.nct;
  float u = (lr - (d.lr0 + cr * dlr)) / dlr * kPatch, v = (t - (d.t0 + ct * dt)) / dt * kPatch;
  u = u < 0.0f ? 0.0f : (u > (float)kPatch ? (float)kPatch : u);
  v = v < 0.0f ? 0.0f : (v > (float)kPatch ? (float)kPatch : v);
  int i = (int)u, j = (int)v;
  i = i > kPatch - 1 ? kPatch - 1 : i;
  j = j > kPatch - 1 ? kPatch - 1 : j;
  const float fu = u - i, fv = v - j;
  const float *p = patch + j * (kPatch + 1) + i;
  const float a = p[0] + fu * (p[1] - p[0]), b = p[kPatch + 1] + fu * (p[kPatch + 2] - p[kPatch + 1]);
  return a + fv * (b - a);
}

template <typename R>
__host__ __device__ __forceinline__ void raw_features(R r, R t, float *raw) {
  const float st = sinf((float)t);
  raw[0] = logf((float)r);
  raw[1] = (float)r * st;
  raw[2] = st;
}

template <typename R>
__host__ __device__ __forceinline__ void features_of(const Domain &d, R r, R t, float *f, bool &inside, int &cell) {
  float raw[3];
  raw_features(r, t, raw);
  for (int k = 0; k < 3; k++) f[k] = (raw[k] - d.fmid[k]) / d.fhalf[k];
  const float lr = raw[0], tt = (float)t;
  inside = lr >= d.lr0 && lr <= d.lr1 && tt >= d.t0 && tt <= d.t1;
  int cr = (int)((lr - d.lr0) / (d.lr1 - d.lr0) * d.ncr), ct = (int)((tt - d.t0) / (d.t1 - d.t0) * d.nct);
  cr = cr < 0 ? 0 : (cr >= d.ncr ? d.ncr - 1 : cr);
  ct = ct < 0 ? 0 : (ct >= d.nct ? d.nct - 1 : ct);
  cell = ct * d.ncr + cr;
}

/* Fills the solid angle of every queued estimator event: the network on the
 * tensor cores for 128 events per tile, the tabulated integrator in flagged
 * cells, zero below the box's lowest theta (as the grid path).  Events
 * outside the box are appended to fb_list for omega_fallback_kernel. */
template <typename R>
__global__ void __launch_bounds__(kFwdThreads, 1) omega_kernel(const unsigned char *packed, const float *theta, Domain dom,
                                                       const unsigned char *flags, const DevBundle<R> *bundles,
                                                       int n_cfg, VrEvent<R> *ev, const unsigned long long *count,
                                                       long long cap, unsigned long long *fallbacks, int *fb_list,
                                                       unsigned long long *fb_count, const int *patch_of,
                                                       const float *patches, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  FwdCtx c;
  fwd_setup(sm, packed, theta, c);
  const long long n = (long long)*count < cap ? (long long)*count : cap;
  bool failed = false;
  for (long long tile = (long long)blockIdx.x * kGroups + c.g; tile * 128 < n; tile += (long long)gridDim.x * kGroups) {
    const long long i = tile * 128 + c.row;
    const bool valid = i < n;
    const R r = valid ? ev[i].sa_r : (R)1, t = valid ? ev[i].sa_t : (R)dom.tmin;
    float f[NIN], y;
    bool inside;
    int cell;
    features_of(dom, r, t, f, inside, cell);
    if (!fwd_tile(sm, c, f, y)) {
      failed = true;
      break;
    }
    /* events of a batch carry their configuration; those of configurations
     * served by the grid were already weighted in transport */
    bool apply = false, need_fb = false;
    R omega = (R)0;
    if (valid) {
      const int cfg = ev[i].cfg;
      if (cfg < 0 || cfg >= n_cfg) {
        atomicExch(err, 2);
      } else if (bundles[cfg].use_surrogate) {
        if (!(t >= (R)dom.tmin)) {
          apply = true;
        } else if (!inside) {
          need_fb = true;
        } else if (flags[cell]) {
          const int pc = patch_of[cell];
          if (pc >= 0) {
            omega = (R)patch_omega(dom, patches + (size_t)pc * kPatchNodes, logf((float)r), (float)t, cell);
            apply = true;
          } else {
            need_fb = true;
          }
        } else {
          const float o = __expf(y) - dom.eps;
          omega = (R)(o > 0.0f ? o : 0.0f);
          apply = true;
        }
      }
    }
    /* warp-aggregated append to the integrator's list */
    const unsigned fb = __ballot_sync(0xffffffffu, need_fb);
    if (fb) {
      const int lane = threadIdx.x & 31, leader = __ffs(fb) - 1;
      unsigned long long base = 0;
      if (lane == leader) {
        base = atomicAdd(fb_count, (unsigned long long)__popc(fb));
        atomicAdd(fallbacks, (unsigned long long)__popc(fb));
      }
      base = __shfl_sync(0xffffffffu, base, leader);
      const unsigned long long pos = base + __popc(fb & ((1u << lane) - 1u));
      if (need_fb && (long long)pos < cap) fb_list[pos] = (int)i;
    }
    if (apply) {
      ev[i].pR *= omega;
      ev[i].pC *= omega;
      ev[i].pdir_fluo *= omega;
    }
  }
  if (failed && c.row == 0) atomicExch(err, 1);
  fwd_teardown(c);
}

/* The integrator for the events omega_kernel could not serve: one warp per
 * event, lane l taking cone samples l, l + 32, ... of the event's own stream
 * (seed, id, 0x80000000 | n) -- sample i is Philox block i of that stream,
 * so the hit count and the solid angle are those of the serial off-grid
 * integral of the grid path (single_solid_angle). */
template <typename R>
__global__ void __launch_bounds__(256) omega_fallback_kernel(const DevBundle<R> *bundles, int n_cfg, VrEvent<R> *ev,
                                                             const int *fb_list, const unsigned long long *fb_count,
                                                             long long cap) {
  const int lane = threadIdx.x & 31;
  const long long n = (long long)*fb_count < cap ? (long long)*fb_count : cap;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += warps) {
    const int i = fb_list[w];
    if (i < 0 || (long long)i >= cap) continue;
    const int cfg = ev[i].cfg;
    if (cfg < 0 || cfg >= n_cfg) continue;
    const DevBundle<R> &b = bundles[cfg];
    const SaGeom g{b.det_radius, b.coll_radius, b.coll_height, b.coll_present};
    const uint64_t id = (uint64_t)ev[i].id;
    const uint32_t stream = 0x80000000u | (uint32_t)ev[i].n;
    R cfca, fcsa, st, ct, py, pz;
    bool outside;
    int hits = 0;
    const bool live = sa_setup<R>(g, ev[i].sa_r, ev[i].sa_t, cfca, fcsa, st, ct, py, pz, outside);
    if (live) {
      for (int s = lane; s < b.sa_hits; s += 32) {
        xmi_u32x4 c;
        c.v[0] = (uint32_t)s;
        c.v[1] = stream;
        c.v[2] = (uint32_t)id;
        c.v[3] = (uint32_t)(id >> 32);
        const xmi_u32x4 o = xmi_philox4x32_10(c, (uint32_t)b.seed, (uint32_t)(b.seed >> 32));
        R u1, u2;
        cone_draws(o, u1, u2);
        hits += sa_sample<R>(g, cfca, st, ct, py, pz, outside, u1, u2);
      }
    }
    hits = __reduce_add_sync(0xffffffffu, hits);
    if (lane == 0) {
      const R omega = live ? fcsa * (R)hits / (R)b.sa_hits : (R)0;
      ev[i].pR *= omega;
      ev[i].pC *= omega;
      ev[i].pdir_fluo *= omega;
    }
  }
}

/* the queued events whose point lay off the solid-angle grid (sa_pending),
 * appended (warp-aggregated) to fb_list for omega_fallback_kernel */
template <typename R>
__global__ void __launch_bounds__(256) collect_pending_kernel(const VrEvent<R> *ev, const unsigned long long *count,
                                                              long long cap, int *fb_list,
                                                              unsigned long long *fb_count) {
  const long long n = (long long)*count < cap ? (long long)*count : cap;
  const int lane = threadIdx.x & 31;
  for (long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; base < n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long i = base + lane;
    const bool pend = i < n && ev[i].sa_pending != 0;
    const unsigned m = __ballot_sync(0xffffffffu, pend);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    unsigned long long pos = 0;
    if (lane == leader) pos = atomicAdd(fb_count, (unsigned long long)__popc(m));
    pos = __shfl_sync(0xffffffffu, pos, leader) + __popc(m & ((1u << lane) - 1u));
    if (pend && (long long)pos < cap) fb_list[pos] = (int)i;
  }
}

/* ---------------- training ---------------- */
/* transposed hidden weights W_l^T (l = 1..3) as K-major tiles: element
 * (in, out) = W_l[out][in]; the B operand of dX = dZ W_l */
__global__ void pack_weights_t(const float *theta, unsigned char *packed_t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3 * H * H) {
    const int l = 1 + i / (H * H), r = i % (H * H), o = r / H, k = r % H;
    *(__nv_bfloat16 *)(packed_t + (l - 1) * WL_BYTES + umma::kmajor_offset(k, o, H)) =
        __float2bfloat16_rn(theta[off_w(l) + o * H + k]);
  }
}

/* shared-memory plan of the training kernel */
constexpr int TR_SW = 0;                  /* weight tile W_l (forward) or W_l^T (backward) */
constexpr int TR_SA = TR_SW + WL_BYTES;   /* activations (forward) / dZ rows (backward) */
constexpr int TR_SDT = TR_SA + WL_BYTES;  /* dZ^T (A operand of dW) */
constexpr int TR_SB = TR_SDT + WL_BYTES;  /* a_l^T (B operand of dW) */
constexpr int TR_SX0 = TR_SB + WL_BYTES;  /* input tile [128 x 16] */
constexpr int TR_BIAS = TR_SX0 + H * KIN * 2;
constexpr int TR_WO = TR_BIAS + 4 * H * 4;
constexpr int TR_G = TR_WO + H * 4;       /* per-CTA partial gradients of b_0..b_3, w_o, b_o */
constexpr int TR_NG = 4 * H + H + 1;
constexpr int TR_BAR = TR_G + ((TR_NG * 4 + 15) / 16) * 16;
constexpr int TR_TOTAL = TR_BAR + 16;
static_assert(TR_TOTAL <= 227 * 1024, "training kernel shared memory");

/* per-CTA global scratch: pre-activations Z_l^T [4][128 units][128 rows] FP32
 * and input activations a_l^T as K-major tiles [4][32 KB] */
constexpr size_t TR_SCRATCH_Z = (size_t)4 * H * H * 4;
constexpr size_t TR_SCRATCH = TR_SCRATCH_Z + (size_t)4 * WL_BYTES;

__device__ __forceinline__ void copy_tile(unsigned char *dst, const unsigned char *src, int bytes) {
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) ((uint4 *)dst)[i] = ((const uint4 *)src)[i];
}

__device__ __forceinline__ float dsilu(float z) {
  const float s = sigmoid_fast(z);
  return s * (1.0f + z * (1.0f - s));
}

/* issues the MMAs of one GEMM: D (+)= A[128 x K] B[N x K]^T, K = 16 ksteps */
__device__ __forceinline__ void gemm_issue(uint32_t d, uint32_t a, uint32_t a_sbo, uint32_t b, uint32_t b_sbo,
                                           int ksteps, uint32_t idesc) {
  for (int kk = 0; kk < ksteps; kk++)
    umma::mma_bf16(d, umma::smem_desc(a + kk * 256, 128, a_sbo), umma::smem_desc(b + kk * 256, 128, b_sbo), idesc,
                   kk > 0);
}

/* One gradient pass: each CTA takes the 128-row tiles tile0 + blockIdx.x,
 * tile0 + blockIdx.x + gridDim.x, ... below n_tiles_used, runs forward and
 * backward, and adds the gradient of sum((y - t)^2) * inv_batch to grad
 * (FP32 atomics) and sum((y - t)^2) to *loss. */
__global__ void __launch_bounds__(128, 1) train_kernel(const unsigned char *packed, const unsigned char *packed_t,
                                                       const float *theta, const float *features,
                                                       const float *targets, int n, int tile0, int n_tiles_used,
                                                       float inv_batch, unsigned char *scratch, float *grad,
                                                       double *loss, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5;
  uint64_t *mbar = (uint64_t *)(sm + TR_BAR);
  uint32_t *tmem_slot = (uint32_t *)(sm + TR_BAR + 8);
  float *bias = (float *)(sm + TR_BIAS), *wo = (float *)(sm + TR_WO), *g = (float *)(sm + TR_G);
  float *zt = (float *)(scratch + (size_t)blockIdx.x * TR_SCRATCH);
  unsigned char *at = scratch + (size_t)blockIdx.x * TR_SCRATCH + TR_SCRATCH_Z;

  for (int i = tid; i < H; i += blockDim.x) {
    bias[i] = theta[OFF_B0 + i];
    for (int l = 1; l <= 3; l++) bias[l * H + i] = theta[off_b(l) + i];
    wo[i] = theta[OFF_WO + i];
  }
  for (int i = tid; i < TR_NG; i += blockDim.x) g[i] = 0.0f;
  for (int i = tid; i < H * KIN * 2 / 16; i += blockDim.x) ((uint4 *)(sm + TR_SX0))[i] = make_uint4(0, 0, 0, 0);
  const float bo = theta[OFF_BO];
  if (warp == 0) umma::tmem_alloc(tmem_slot, 256);
  if (tid == 0) {
    umma::mbar_init(mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_proxy_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t d1 = tmem, d2 = tmem + 128; /* dW accumulators, forward / dX accumulators */
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
  const uint32_t s_w = umma::smem_u32(sm + TR_SW), s_a = umma::smem_u32(sm + TR_SA),
                 s_dt = umma::smem_u32(sm + TR_SDT), s_b = umma::smem_u32(sm + TR_SB),
                 s_x0 = umma::smem_u32(sm + TR_SX0);
  uint32_t phase = 0;
  bool failed = false;

  /* issue (thread 0) after the CTA's operand writes, then wait for completion */
  auto run_mma = [&](auto &&issue) -> bool {
    umma::fence_proxy_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after_sync();
      issue();
      umma::mma_commit(mbar);
    }
    const bool ok = umma::mbar_wait(mbar, phase);
    phase ^= 1u;
    const bool any_fail = __syncthreads_or(!ok);
    umma::fence_after_sync();
    return !any_fail;
  };

  for (int tile = tile0 + blockIdx.x; tile < tile0 + n_tiles_used && !failed; tile += gridDim.x) {
    const int row = tile * 128 + tid;
    const bool valid = row < n;
    /* ---- forward ---- */
    for (int k = 0; k < NIN; k++) {
      const __nv_bfloat16 v = __float2bfloat16_rn(valid ? features[(size_t)row * NIN + k] : 0.0f);
      *(__nv_bfloat16 *)(sm + TR_SX0 + umma::kmajor_offset(tid, k, KIN)) = v;
      *(__nv_bfloat16 *)(at + umma::kmajor_offset(k, tid, H)) = v;
    }
    for (int k = NIN; k < KIN; k++) *(__nv_bfloat16 *)(at + umma::kmajor_offset(k, tid, H)) = __float2bfloat16_rn(0.0f);
    float y = bo;
    {
      /* layer 0 in FP32 on the CUDA cores (as the forward kernel) */
      float f[NIN];
      for (int k = 0; k < NIN; k++) f[k] = valid ? features[(size_t)row * NIN + k] : 0.0f;
      for (int j = 0; j < H; j++) {
        const float z = bias[j] + theta[OFF_W0 + j * NIN] * f[0] + theta[OFF_W0 + j * NIN + 1] * f[1] +
                        theta[OFF_W0 + j * NIN + 2] * f[2];
        zt[(size_t)j * H + tid] = z;
        const __nv_bfloat16 a = __float2bfloat16_rn(silu(z));
        *(__nv_bfloat16 *)(sm + TR_SA + umma::kmajor_offset(tid, j, H)) = a;
        *(__nv_bfloat16 *)(at + (size_t)WL_BYTES + umma::kmajor_offset(j, tid, H)) = a;
      }
    }
    for (int l = 1; l < 4 && !failed; l++) {
      copy_tile(sm + TR_SW, packed + W0_BYTES + (l - 1) * WL_BYTES, WL_BYTES);
      const uint32_t idesc = umma::idesc_bf16_f32(128, 128);
      if (!run_mma([&] { gemm_issue(d2, s_a, 2048, s_w, 2048, H / 16, idesc); })) {
        failed = true;
        break;
      }
#pragma unroll 1
      for (int c = 0; c < H / 32; c++) {
        float v[32];
        umma::tmem_ld_32x32b_x32(d2 + lane_off + c * 32, v);
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const int col = c * 32 + j;
          const float z = v[j] + bias[l * H + col];
          zt[((size_t)l * H + col) * H + tid] = z;
          const float h = silu(z);
          if (l < 3) {
            const __nv_bfloat16 a = __float2bfloat16_rn(h);
            *(__nv_bfloat16 *)(sm + TR_SA + umma::kmajor_offset(tid, col, H)) = a;
            *(__nv_bfloat16 *)(at + (size_t)(l + 1) * WL_BYTES + umma::kmajor_offset(col, tid, H)) = a;
          } else {
            y += h * wo[col];
          }
        }
      }
    }
    if (failed) break;
    /* ---- loss and output layer ---- */
    const float diff = valid ? y - targets[row] : 0.0f;
    const float dy = 2.0f * diff * inv_batch;
    atomicAdd(loss, (double)diff * (double)diff);
    atomicAdd(&g[4 * H + H], dy);
    for (int col = 0; col < H; col++) {
      const float z = zt[((size_t)3 * H + col) * H + tid];
      atomicAdd(&g[4 * H + col], dy * silu(z));
      const float dz = dy * wo[col] * dsilu(z);
      atomicAdd(&g[3 * H + col], dz);
      const __nv_bfloat16 bz = __float2bfloat16_rn(dz);
      *(__nv_bfloat16 *)(sm + TR_SA + umma::kmajor_offset(tid, col, H)) = bz;
      *(__nv_bfloat16 *)(sm + TR_SDT + umma::kmajor_offset(col, tid, H)) = bz;
    }
    /* ---- hidden layers, l = 3 .. 0: dW_l = dZ_l^T a_l, dZ_{l-1} = (dZ_l W_l) * SiLU'(Z_{l-1}) ---- */
    for (int l = 3; l >= 0 && !failed; l--) {
      const int nin = l == 0 ? KIN : H;
      copy_tile(sm + TR_SB, at + (size_t)l * WL_BYTES, l == 0 ? KIN * H * 2 : WL_BYTES);
      if (l > 0) copy_tile(sm + TR_SW, packed_t + (l - 1) * WL_BYTES, WL_BYTES);
      if (!run_mma([&] {
            gemm_issue(d1, s_dt, 2048, s_b, 2048, H / 16, umma::idesc_bf16_f32(128, nin));
            if (l > 0) gemm_issue(d2, s_a, 2048, s_w, 2048, H / 16, umma::idesc_bf16_f32(128, 128));
          })) {
        failed = true;
        break;
      }
      /* dW_l rows: thread = output unit */
#pragma unroll 1
      for (int c = 0; c < (nin + 31) / 32; c++) {
        float v[32];
        umma::tmem_ld_32x32b_x32(d1 + lane_off + c * 32, v);
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const int col = c * 32 + j;
          if (l == 0) {
            if (col < NIN) atomicAdd(&grad[OFF_W0 + tid * NIN + col], v[j]);
          } else {
            atomicAdd(&grad[off_w(l) + tid * H + col], v[j]);
          }
        }
      }
      if (l > 0) {
        /* dZ_{l-1} rows: thread = sample */
        __syncthreads(); /* every dZ_l operand read by the MMAs above is complete; safe to overwrite */
#pragma unroll 1
        for (int c = 0; c < H / 32; c++) {
          float v[32];
          umma::tmem_ld_32x32b_x32(d2 + lane_off + c * 32, v);
#pragma unroll
          for (int j = 0; j < 32; j++) {
            const int col = c * 32 + j;
            const float dz = valid ? v[j] * dsilu(zt[((size_t)(l - 1) * H + col) * H + tid]) : 0.0f;
            atomicAdd(&g[(l - 1) * H + col], dz);
            const __nv_bfloat16 bz = __float2bfloat16_rn(dz);
            *(__nv_bfloat16 *)(sm + TR_SA + umma::kmajor_offset(tid, col, H)) = bz;
            *(__nv_bfloat16 *)(sm + TR_SDT + umma::kmajor_offset(col, tid, H)) = bz;
          }
        }
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < TR_NG; i += blockDim.x) {
    const float v = g[i];
    if (v == 0.0f) continue;
    int at_index;
    if (i < 4 * H) at_index = (i < H ? OFF_B0 : off_b(i / H)) + i % H;
    else if (i < 5 * H) at_index = OFF_WO + (i - 4 * H);
    else at_index = OFF_BO;
    atomicAdd(&grad[at_index], v);
  }
  if (failed && tid == 0) atomicExch(err, 1);
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

/* Adam step on the FP32 master parameters; clears the gradient */
__global__ void adam_kernel(float *theta, float *m, float *v, float *grad, float lr, float b1, float b2, float eps,
                            float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const float gi = grad[i];
  grad[i] = 0.0f;
  const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  theta[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

}  // namespace mlp
}  // namespace xmi

extern "C" {

int xmi_mlp_nparam(void) { return xmi::mlp::NPARAM; }

namespace {
/* device state of one training / gradient session */
struct MlpTrainer {
  float *theta = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *feat = nullptr, *targ = nullptr;
  unsigned char *packed = nullptr, *packed_t = nullptr, *scratch = nullptr;
  double *loss = nullptr;
  int *err = nullptr;
  int n = 0, grid = 1;
  bool alloc(int n_rows, const float *theta_h, const float *feat_h, const float *targ_h) {
    using namespace xmi::mlp;
    n = n_rows;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (n + 127) / 128;
    grid = tiles < sms ? tiles : sms;
    bool ok = cudaMalloc(&theta, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&m, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&v, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&grad, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&feat, sizeof(float) * 3 * (size_t)n) == cudaSuccess &&
              cudaMalloc(&targ, sizeof(float) * (size_t)n) == cudaSuccess &&
              cudaMalloc(&packed, PACK_BYTES) == cudaSuccess && cudaMalloc(&packed_t, 3 * WL_BYTES) == cudaSuccess &&
              cudaMalloc(&scratch, TR_SCRATCH * (size_t)grid) == cudaSuccess &&
              cudaMalloc(&loss, sizeof(double)) == cudaSuccess && cudaMalloc(&err, sizeof(int)) == cudaSuccess;
    if (!ok) return false;
    cudaMemcpy(theta, theta_h, sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
    cudaMemcpy(feat, feat_h, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(targ, targ_h, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemset(m, 0, sizeof(float) * NPARAM);
    cudaMemset(v, 0, sizeof(float) * NPARAM);
    cudaMemset(grad, 0, sizeof(float) * NPARAM);
    cudaMemset(err, 0, sizeof(int));
    cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TR_TOTAL);
    return true;
  }
  /* gradient of the mean squared error over tiles [tile0, tile0 + ntiles) */
  void grad_pass(int tile0, int ntiles, int rows) {
    using namespace xmi::mlp;
    pack_weights<<<(3 * H * H + 255) / 256, 256>>>(theta, packed);
    pack_weights_t<<<(3 * H * H + 255) / 256, 256>>>(theta, packed_t);
    cudaMemsetAsync(loss, 0, sizeof(double));
    const int g = ntiles < grid ? ntiles : grid;
    train_kernel<<<g, 128, TR_TOTAL>>>(packed, packed_t, theta, feat, targ, n, tile0, ntiles, 1.0f / (float)rows,
                                       scratch, grad, loss, err);
  }
  void release() {
    cudaFree(theta); cudaFree(m); cudaFree(v); cudaFree(grad); cudaFree(feat); cudaFree(targ);
    cudaFree(packed); cudaFree(packed_t); cudaFree(scratch); cudaFree(loss); cudaFree(err);
  }
};

/* Adam over the trainer's rows (in order): one 128-row tile per SM per step,
 * learning rate decaying by a cosine from lr to lr/100 */
bool train_loop(MlpTrainer &tr, int epochs, float lr, double *loss_per_epoch);

bool finish(MlpTrainer &tr, const char *what) {
  cudaError_t e = cudaDeviceSynchronize();
  int h_err = 0;
  if (e == cudaSuccess) cudaMemcpy(&h_err, tr.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    xmi_set_error("%s: %s", what, cudaGetErrorString(e));
    return false;
  }
  if (h_err) {
    xmi_set_error("%s: tensor-core wait ran out", what);
    return false;
  }
  return true;
}
}  // namespace

/* Gradient of the mean squared error of the network over n rows (host
 * arrays): grad[NPARAM], *loss = mean squared error.  For the checks of the
 * tensor-core backward pass. */
int xmi_gpu_mlp_grad(const float *theta, int n, const float *features, const float *targets, float *grad,
                     double *loss) {
  using namespace xmi::mlp;
  if (!theta || !features || !targets || !grad || n < 1) {
    xmi_set_error("xmi_gpu_mlp_grad: invalid arguments");
    return 0;
  }
  MlpTrainer tr;
  bool ok = tr.alloc(n, theta, features, targets);
  if (ok) {
    tr.grad_pass(0, (n + 127) / 128, n);
    ok = finish(tr, "xmi_gpu_mlp_grad");
    if (ok) {
      double l = 0.0;
      cudaMemcpy(grad, tr.grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
      cudaMemcpy(&l, tr.loss, sizeof(double), cudaMemcpyDeviceToHost);
      if (loss) *loss = l / n;
    }
  } else {
    xmi_set_error("xmi_gpu_mlp_grad: cudaMalloc failed");
  }
  tr.release();
  return ok ? 1 : 0;
}

/* Adam training of the network on n rows (host arrays), in place on theta:
 * each step takes one 128-row tile per SM (the rows are used in order, so
 * shuffle them beforehand), epochs passes over the data, learning rate lr
 * decaying by a cosine to lr/100.  loss_per_epoch[epochs] (may be NULL)
 * receives the mean squared error seen during each epoch. */
int xmi_gpu_mlp_train(float *theta, int n, const float *features, const float *targets, int epochs, float lr,
                      double *loss_per_epoch) {
  using namespace xmi::mlp;
  if (!theta || !features || !targets || n < 1 || epochs < 1) {
    xmi_set_error("xmi_gpu_mlp_train: invalid arguments");
    return 0;
  }
  MlpTrainer tr;
  bool ok = tr.alloc(n, theta, features, targets);
  if (!ok) xmi_set_error("xmi_gpu_mlp_train: cudaMalloc failed");
  ok = ok && train_loop(tr, epochs, lr, loss_per_epoch);
  if (ok) cudaMemcpy(theta, tr.theta, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
  tr.release();
  return ok ? 1 : 0;
}

/* Network outputs for n feature rows with the FP32 parameter vector theta
 * (host arrays); for tests of the tensor-core kernels. */
int xmi_gpu_mlp_forward(const float *theta, int n, const float *features, float *out) {
  using namespace xmi::mlp;
  if (!theta || !features || !out || n < 1) {
    xmi_set_error("xmi_gpu_mlp_forward: invalid arguments");
    return 0;
  }
  float *d_theta = nullptr, *d_feat = nullptr, *d_out = nullptr;
  unsigned char *d_pack = nullptr;
  int *d_err = nullptr, h_err = 0;
  bool ok = cudaMalloc(&d_theta, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&d_feat, sizeof(float) * 3 * (size_t)n) == cudaSuccess &&
            cudaMalloc(&d_out, sizeof(float) * (size_t)n) == cudaSuccess &&
            cudaMalloc(&d_pack, PACK_BYTES) == cudaSuccess && cudaMalloc(&d_err, sizeof(int)) == cudaSuccess;
  if (ok) {
    cudaMemcpy(d_theta, theta, sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
    cudaMemcpy(d_feat, features, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemset(d_err, 0, sizeof(int));
    pack_weights<<<(3 * H * H + 255) / 256, 256>>>(d_theta, d_pack);
    cudaFuncSetAttribute(forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (n + 127) / 128;
    forward_kernel<<<tiles < sms ? tiles : sms, kFwdThreads, SM_TOTAL>>>(d_pack, d_theta, d_feat, d_out, n, d_err);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      xmi_set_error("xmi_gpu_mlp_forward: %s", cudaGetErrorString(e));
      ok = false;
    } else {
      cudaMemcpy(out, d_out, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost);
      cudaMemcpy(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost);
      if (h_err) {
        xmi_set_error("xmi_gpu_mlp_forward: tensor-core wait ran out");
        ok = false;
      }
    }
  } else {
    xmi_set_error("xmi_gpu_mlp_forward: cudaMalloc failed");
  }
  cudaFree(d_theta);
  cudaFree(d_feat);
  cudaFree(d_out);
  cudaFree(d_pack);
  cudaFree(d_err);
  return ok ? 1 : 0;
}

}  // extern "C"

namespace {
bool train_loop(MlpTrainer &tr, int epochs, float lr, double *loss_per_epoch) {
  using namespace xmi::mlp;
  const int n = tr.n, tiles = (n + 127) / 128;
  const int steps_per_epoch = (tiles + tr.grid - 1) / tr.grid;
  const int total = steps_per_epoch * epochs;
  int step = 0;
  bool ok = true;
  for (int ep = 0; ok && ep < epochs; ep++) {
    double ep_loss = 0.0;
    for (int s = 0; s < steps_per_epoch; s++, step++) {
      const int tile0 = s * tr.grid, nt = tile0 + tr.grid <= tiles ? tr.grid : tiles - tile0;
      const int rows = (tile0 + nt) * 128 <= n ? nt * 128 : n - tile0 * 128;
      tr.grad_pass(tile0, nt, rows);
      const float frac = (float)step / (float)(total > 1 ? total - 1 : 1);
      const float lr_t = lr * (0.01f + 0.99f * 0.5f * (1.0f + cosf(3.14159265f * frac)));
      const float bc1 = 1.0f - powf(0.9f, (float)(step + 1)), bc2 = 1.0f - powf(0.999f, (float)(step + 1));
      adam_kernel<<<(NPARAM + 255) / 256, 256>>>(tr.theta, tr.m, tr.v, tr.grad, lr_t, 0.9f, 0.999f, 1e-8f, bc1, bc2);
      double l = 0.0;
      cudaMemcpy(&l, tr.loss, sizeof(double), cudaMemcpyDeviceToHost);
      ep_loss += l;
    }
    if (loss_per_epoch) loss_per_epoch[ep] = ep_loss / n;
    ok = finish(tr, "surrogate training");
  }
  return ok;
}

/* trained surrogate of one input's solid-angle grid */
struct SurrogateState {
  std::atomic<int> refs{1}; /* input handles sharing this network */
  xmi::SaGeom geom;         /* detector and collimator it was trained for */
  xmi::mlp::Domain dom;
  std::vector<float> theta;
  float *theta_d = nullptr;
  unsigned char *packed_d = nullptr, *flags_d = nullptr;
  int *patch_of_d = nullptr;  /* [ncell]: patch of a flagged cell, -1 otherwise */
  float *patches_d = nullptr; /* [n_patch][kPatchNodes] */
  int n_patch = 0;
  double report[6] = {0, 0, 0, 0, 0, 0};
};

/* network outputs on the device for n feature rows already on the device */
bool device_forward(const SurrogateState &sg, const float *feat_d, float *out_d, int n, int *err_d) {
  using namespace xmi::mlp;
  cudaFuncSetAttribute(forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = (n + 127) / 128;
  forward_kernel<<<tiles < sms ? tiles : sms, kFwdThreads, SM_TOTAL>>>(sg.packed_d, sg.theta_d, feat_d, out_d, n, err_d);
  return cudaDeviceSynchronize() == cudaSuccess;
}
}  // namespace

extern "C" {

void xmi_surrogate_free(void *p) {
  SurrogateState *sg = (SurrogateState *)p;
  if (!sg || --sg->refs > 0) return;
  cudaFree(sg->theta_d);
  cudaFree(sg->packed_d);
  cudaFree(sg->flags_d);
  cudaFree(sg->patch_of_d);
  cudaFree(sg->patches_d);
  delete sg;
}

/* Trains the solid-angle surrogate of an initialised input handle (see
 * xmi_gpu_build_surrogate in the public header for the procedure). */
constexpr int kCells = 32, kCheckPerCell = 16, kCheckPoints = kCells * kCells * kCheckPerCell;
constexpr int kPatchHits = 1 << 16; /* integrator samples per node of a flagged cell's table */

static int build_from_points(xmi_inputFPtr in, std::vector<double> &r_h, std::vector<double> &t_h, int n_train,
                             int hits_train, int epochs, int hits_check, double *report,
                             std::chrono::steady_clock::time_point t_start);

static bool surrogate_device_ok() {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    xmi_set_error("no CUDA device available: the engine has no CPU fallback");
    return false;
  }
  return true;
}

int xmi_gpu_build_surrogate(xmi_inputFPtr in, int n_train, int hits_train, int epochs, int hits_check,
                            double *report) {
  if (!in || !in->initialized || n_train < 128 || hits_train < 1 || epochs < 1 || hits_check < 1) {
    xmi_set_error("xmi_gpu_build_surrogate: invalid arguments");
    return 0;
  }
  if (!surrogate_device_ok()) return 0;
  const auto t_start = std::chrono::steady_clock::now();
  const int n_check = kCheckPoints;

  /* training and checking points uniform over the sample volume: the slab
   * between the first and last layer planes, within kLateral of the beam
   * axis (the z axis), mapped to the (r, theta) of the solid-angle grid.
   * The layer plane at offset h along the sample normal n (x . n = h) meets
   * the beam at (0, 0, h / n_z). */
  std::mt19937_64 rng(0x5EED0004ull);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  std::vector<double> r_h(n_train + 2 * n_check), t_h(n_train + 2 * n_check);
  {
    const double kLateral = 2.0; /* cm */
    const double *nv = in->n_sample;
    double e1[3] = {1.0, 0.0, 0.0};
    if (std::fabs(nv[0]) > 0.9) e1[0] = 0.0, e1[1] = 1.0;
    const double d1 = e1[0] * nv[0] + e1[1] * nv[1] + e1[2] * nv[2];
    for (int k = 0; k < 3; k++) e1[k] -= d1 * nv[k];
    const double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int k = 0; k < 3; k++) e1[k] /= l1;
    const double e2[3] = {nv[1] * e1[2] - nv[2] * e1[1], nv[2] * e1[0] - nv[0] * e1[2], nv[0] * e1[1] - nv[1] * e1[0]};
    const int nl = in->input->composition->n_layers;
    const double h0 = in->layer_zbeg[0] * nv[2], h1 = in->layer_zend[nl - 1] * nv[2];
    for (int i = 0; i < n_train + n_check; i++) {
      const double a = (2.0 * u01(rng) - 1.0) * kLateral, b = (2.0 * u01(rng) - 1.0) * kLateral;
      const double h = h0 + (h1 - h0) * u01(rng);
      double x[3], dv[3];
      for (int k = 0; k < 3; k++) x[k] = a * e1[k] + b * e2[k];
      x[2] += h / nv[2];
      for (int k = 0; k < 3; k++) dv[k] = x[k] - in->p_det[k];
      const double r = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
      double tt = std::acos((dv[0] * in->n_det[0] + dv[1] * in->n_det[1] + dv[2] * in->n_det[2]) / r);
      if (tt > M_PI / 2.0) tt = M_PI - tt;
      r_h[i] = r;
      t_h[i] = M_PI / 2.0 - tt;
    }
  }
  return build_from_points(in, r_h, t_h, n_train, hits_train, epochs, hits_check, report, t_start);
}

int xmi_gpu_build_surrogate_points(xmi_inputFPtr in, int n_points, const double *r, const double *theta,
                                   int hits_train, int epochs, int hits_check, double *report) {
  if (!in || !in->initialized || !r || !theta || n_points < kCheckPoints + 128 || hits_train < 1 || epochs < 1 ||
      hits_check < 1) {
    xmi_set_error("xmi_gpu_build_surrogate_points: invalid arguments (at least %d points)", kCheckPoints + 128);
    return 0;
  }
  if (!surrogate_device_ok()) return 0;
  const auto t_start = std::chrono::steady_clock::now();
  /* fixed shuffle; the first kCheckPoints check, the rest train (points are
   * stored training first) */
  std::vector<int> perm(n_points);
  for (int i = 0; i < n_points; i++) perm[i] = i;
  std::mt19937_64 rng(0x5EED0006ull);
  std::shuffle(perm.begin(), perm.end(), rng);
  const int n_train = n_points - kCheckPoints;
  std::vector<double> r_h(n_points + kCheckPoints), t_h(n_points + kCheckPoints);
  for (int i = 0; i < n_points; i++) {
    const int src = perm[i], dst = i < kCheckPoints ? n_train + i : i - kCheckPoints;
    r_h[dst] = r[src];
    t_h[dst] = theta[src];
  }
  return build_from_points(in, r_h, t_h, n_train, hits_train, epochs, hits_check, report, t_start);
}

/* Trains the network on points [0, n_train) of r_h/t_h (targets from the
 * FP32 integrator) and checks it on the next kCheckPoints (FP64 integrator,
 * twice); r_h/t_h hold n_train + 2 kCheckPoints entries. */
static int build_from_points(xmi_inputFPtr in, std::vector<double> &r_h, std::vector<double> &t_h, int n_train,
                             int hits_train, int epochs, int hits_check, double *report,
                             std::chrono::steady_clock::time_point t_start) {
  using namespace xmi::mlp;
  SurrogateState *sg = new SurrogateState();
  std::vector<double> rv(1024), tv(1024);
  xmi_solid_angle_axes(in, 1024, 1024, rv.data(), tv.data());
  sg->dom.tmin = (float)tv.front();
  sg->dom.ncr = kCells;
  sg->dom.nct = kCells;
  sg->dom.eps = 1e-10f;
  const xmi::SaGeom geom{in->det_radius, in->coll_radius, in->coll_height, in->coll_present};
  sg->geom = geom;
  const int ncell = sg->dom.ncr * sg->dom.nct, n_check = kCheckPoints;
  std::mt19937_64 rng(0x5EED0004ull);
  {
    /* feature scaling and checked box from the training points */
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    float tlo = 1e30f, thi = -1e30f;
    for (int i = 0; i < n_train; i++) {
      float raw[3];
      raw_features(r_h[i], t_h[i], raw);
      for (int k = 0; k < 3; k++) {
        lo[k] = std::min(lo[k], raw[k]);
        hi[k] = std::max(hi[k], raw[k]);
      }
      tlo = std::min(tlo, (float)t_h[i]);
      thi = std::max(thi, (float)t_h[i]);
    }
    for (int k = 0; k < 3; k++) {
      sg->dom.fmid[k] = 0.5f * (lo[k] + hi[k]);
      sg->dom.fhalf[k] = std::max(0.5f * (hi[k] - lo[k]), 1e-6f);
    }
    sg->dom.lr0 = lo[0];
    sg->dom.lr1 = std::max(hi[0], lo[0] + 1e-6f);
    sg->dom.t0 = tlo;
    sg->dom.t1 = std::max(thi, tlo + 1e-6f);
  }
  /* every checking point is integrated twice with independent streams of
   * hits_check / 2 samples: their mean is the reference value and their
   * difference measures its own Monte Carlo noise */
  for (int i = 0; i < n_check; i++) {
    r_h[n_train + n_check + i] = r_h[n_train + i];
    t_h[n_train + n_check + i] = t_h[n_train + i];
  }
  const int half_check = hits_check / 2 > 0 ? hits_check / 2 : 1;
  double *r_d = nullptr, *t_d = nullptr, *o_d = nullptr;
  float *feat_d = nullptr, *pred_d = nullptr;
  int *err_d = nullptr;
  const int ntot = n_train + 2 * n_check;
  bool ok = cudaMalloc(&r_d, sizeof(double) * ntot) == cudaSuccess &&
            cudaMalloc(&t_d, sizeof(double) * ntot) == cudaSuccess &&
            cudaMalloc(&o_d, sizeof(double) * ntot) == cudaSuccess &&
            cudaMalloc(&feat_d, sizeof(float) * 3 * n_check) == cudaSuccess &&
            cudaMalloc(&pred_d, sizeof(float) * n_check) == cudaSuccess &&
            cudaMalloc(&err_d, sizeof(int)) == cudaSuccess;
  std::vector<double> o_h(ntot);
  if (ok) {
    cudaMemcpy(r_d, r_h.data(), sizeof(double) * ntot, cudaMemcpyHostToDevice);
    cudaMemcpy(t_d, t_h.data(), sizeof(double) * ntot, cudaMemcpyHostToDevice);
    cudaMemset(err_d, 0, sizeof(int));
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned long long seed = in->gpu.seed ? in->gpu.seed : 0x5EED0001ull;
    /* training targets: FP32 integrator; checking values: FP64 integrator */
    xmi::solid_angle_points_kernel<float><<<sms * 8, 256>>>(geom, r_d, t_d, n_train, hits_train, seed, o_d);
    xmi::solid_angle_points_kernel<double><<<sms * 8, 256>>>(geom, r_d + n_train, t_d + n_train, n_check,
                                                             half_check, seed ^ 0x9E3779B97F4A7C15ull,
                                                             o_d + n_train);
    xmi::solid_angle_points_kernel<double><<<sms * 8, 256>>>(geom, r_d + n_train + n_check,
                                                             t_d + n_train + n_check, n_check, half_check,
                                                             seed ^ 0xC2B2AE3D27D4EB4Full, o_d + n_train + n_check);
    ok = cudaDeviceSynchronize() == cudaSuccess;
    if (ok) cudaMemcpy(o_h.data(), o_d, sizeof(double) * ntot, cudaMemcpyDeviceToHost);
  }
  if (ok) {
    /* log target log(omega + eps) with eps 1e-4 of the largest training
     * solid angle: relative accuracy where the solid angle matters, and no
     * cliff of 20 units in log space at a collimator's shadow edge */
    double omax = 0.0;
    for (int i = 0; i < n_train; i++) omax = std::max(omax, o_h[i]);
    sg->dom.eps = omax > 0.0 ? (float)(1e-4 * omax) : 1e-10f;
    std::vector<float> feat(3 * (size_t)n_train), targ(n_train);
    for (int i = 0; i < n_train; i++) {
      bool inside;
      int cell;
      features_of(sg->dom, r_h[i], t_h[i], &feat[3 * (size_t)i], inside, cell);
      targ[i] = (float)std::log(o_h[i] + sg->dom.eps);
    }
    sg->theta.resize(NPARAM);
    /* He initialisation, fixed seed */
    std::normal_distribution<double> nrm(0.0, 1.0);
    for (int i = 0; i < NPARAM; i++) sg->theta[i] = 0.0f;
    for (int i = 0; i < H * NIN; i++) sg->theta[OFF_W0 + i] = (float)(nrm(rng) * std::sqrt(2.0 / NIN));
    for (int l = 1; l <= 3; l++)
      for (int i = 0; i < H * H; i++) sg->theta[off_w(l) + i] = (float)(nrm(rng) * std::sqrt(2.0 / H));
    for (int i = 0; i < H; i++) sg->theta[OFF_WO + i] = (float)(nrm(rng) * std::sqrt(1.0 / H));
    double mean = 0.0;
    for (int i = 0; i < n_train; i++) mean += targ[i];
    sg->theta[OFF_BO] = (float)(mean / n_train);
    MlpTrainer tr;
    std::vector<double> hist(epochs);
    ok = tr.alloc(n_train, sg->theta.data(), feat.data(), targ.data()) && train_loop(tr, epochs, 2e-3f, hist.data());
    if (ok) {
      cudaMemcpy(sg->theta.data(), tr.theta, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
      sg->report[3] = hist.back();
    }
    tr.release();
  }
  if (ok) {
    ok = cudaMalloc(&sg->theta_d, sizeof(float) * NPARAM) == cudaSuccess &&
         cudaMalloc(&sg->packed_d, PACK_BYTES) == cudaSuccess && cudaMalloc(&sg->flags_d, ncell) == cudaSuccess;
  }
  if (ok) {
    cudaMemcpy(sg->theta_d, sg->theta.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
    pack_weights<<<(3 * H * H + 255) / 256, 256>>>(sg->theta_d, sg->packed_d);
    std::vector<float> fc(3 * (size_t)n_check);
    for (int i = 0; i < n_check; i++) {
      bool inside;
      int cell;
      features_of(sg->dom, r_h[n_train + i], t_h[n_train + i], &fc[3 * (size_t)i], inside, cell);
    }
    cudaMemcpy(feat_d, fc.data(), sizeof(float) * 3 * n_check, cudaMemcpyHostToDevice);
    ok = device_forward(*sg, feat_d, pred_d, n_check, err_d);
    int h_err = 0;
    cudaMemcpy(&h_err, err_d, sizeof(int), cudaMemcpyDeviceToHost);
    if (h_err) {
      xmi_set_error("xmi_gpu_build_surrogate: tensor-core wait ran out");
      ok = false;
    }
  }
  if (ok) {
    /* cells whose checking points miss the integrator by more than the
     * tolerance are served by the integrator */
    std::vector<float> pred(n_check);
    cudaMemcpy(pred.data(), pred_d, sizeof(float) * n_check, cudaMemcpyDeviceToHost);
    /* per cell: the RMS relative error of the network over its checking
     * points -- relative to omega + eps, as the network's target -- with the
     * reference values' own noise variance (from the two independent
     * integrations) subtracted; cells without checking points (outside the
     * sample volume) are flagged */
    std::vector<double> cell_e2(ncell, 0.0), cell_n2(ncell, 0.0), errs;
    std::vector<int> cell_n(ncell, 0);
    const double eps = sg->dom.eps;
    for (int i = 0; i < n_check; i++) {
      bool inside;
      int cell;
      float f[NIN];
      features_of(sg->dom, r_h[n_train + i], t_h[n_train + i], f, inside, cell);
      if (!inside) continue;
      const double a = o_h[n_train + i], b = o_h[n_train + n_check + i], truth = 0.5 * (a + b);
      const double net = std::max(0.0, std::exp((double)pred[i]) - sg->dom.eps);
      cell_n[cell]++;
      const double e = (net - truth) / (truth + eps), nz = (a - b) / (2.0 * (truth + eps));
      errs.push_back(std::fabs(e));
      cell_e2[cell] += e * e;
      cell_n2[cell] += nz * nz;
    }
    if (errs.empty()) errs.push_back(1.0);
    std::vector<unsigned char> flags(ncell, 0);
    double worst_kept = 0.0;
    const double tol = in->gpu.surrogate_tolerance > 0 ? in->gpu.surrogate_tolerance : 1e-3;
    for (int c = 0; c < ncell; c++) {
      const double err = cell_n[c] > 0 ? std::sqrt(std::max(0.0, (cell_e2[c] - cell_n2[c]) / cell_n[c])) : 1.0;
      flags[c] = (cell_n[c] == 0 || err > tol) ? 1 : 0;
      if (!flags[c]) worst_kept = std::max(worst_kept, err);
    }
    std::vector<double> sorted = errs;
    std::nth_element(sorted.begin(), sorted.begin() + sorted.size() / 2, sorted.end());
    /* share of checking points (drawn like the queries) that land in flagged cells */
    int nflag = 0, ntot = 0;
    for (int i = 0; i < n_check; i++) {
      bool inside;
      int cell;
      float f[NIN];
      features_of(sg->dom, r_h[n_train + i], t_h[n_train + i], f, inside, cell);
      ntot++;
      nflag += (!inside || flags[cell]) ? 1 : 0;
    }
    sg->report[0] = sorted[sorted.size() / 2];
    sg->report[1] = worst_kept;
    sg->report[2] = (double)nflag / (ntot > 0 ? ntot : 1);
    cudaMemcpy(sg->flags_d, flags.data(), ncell, cudaMemcpyHostToDevice);
    /* the tabulated integrator of the flagged cells, FP64, patch_hits
     * samples per node */
    std::vector<int> patch_of(ncell, -1);
    std::vector<double> pr, pt;
    for (int c = 0; c < ncell; c++) {
      if (!flags[c]) continue;
      patch_of[c] = sg->n_patch++;
      const int cr = c % sg->dom.ncr, ct = c / sg->dom.ncr;
      const double dlr = ((double)sg->dom.lr1 - sg->dom.lr0) / sg->dom.ncr;
      const double dt = ((double)sg->dom.t1 - sg->dom.t0) / sg->dom.nct;
      for (int j = 0; j <= kPatch; j++)
        for (int i = 0; i <= kPatch; i++) {
          pr.push_back(std::exp(sg->dom.lr0 + (cr + (double)i / kPatch) * dlr));
          pt.push_back(sg->dom.t0 + (ct + (double)j / kPatch) * dt);
        }
    }
    const int np = (int)pr.size();
    ok = cudaMalloc(&sg->patch_of_d, sizeof(int) * ncell) == cudaSuccess &&
         cudaMalloc(&sg->patches_d, sizeof(float) * (np > 0 ? np : 1)) == cudaSuccess;
    if (ok && np > 0) {
      double *nr_d = nullptr, *nt_d = nullptr, *no_d = nullptr;
      ok = cudaMalloc(&nr_d, sizeof(double) * np) == cudaSuccess &&
           cudaMalloc(&nt_d, sizeof(double) * np) == cudaSuccess &&
           cudaMalloc(&no_d, sizeof(double) * np) == cudaSuccess;
      if (ok) {
        cudaMemcpy(nr_d, pr.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
        cudaMemcpy(nt_d, pt.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const unsigned long long seed = in->gpu.seed ? in->gpu.seed : 0x5EED0001ull;
        xmi::solid_angle_points_kernel<double><<<sms * 8, 256>>>(geom, nr_d, nt_d, np, kPatchHits,
                                                                 seed ^ 0x165667B19E3779F9ull, no_d);
        std::vector<double> po(np);
        ok = cudaDeviceSynchronize() == cudaSuccess &&
             cudaMemcpy(po.data(), no_d, sizeof(double) * np, cudaMemcpyDeviceToHost) == cudaSuccess;
        std::vector<float> pf(po.begin(), po.end());
        if (ok) cudaMemcpy(sg->patches_d, pf.data(), sizeof(float) * np, cudaMemcpyHostToDevice);
      }
      cudaFree(nr_d);
      cudaFree(nt_d);
      cudaFree(no_d);
    }
    if (ok) cudaMemcpy(sg->patch_of_d, patch_of.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice);
  }
  cudaFree(r_d);
  cudaFree(t_d);
  cudaFree(o_d);
  cudaFree(feat_d);
  cudaFree(pred_d);
  cudaFree(err_d);
  if (!ok) {
    if (!*xmi_gpu_last_error()) xmi_set_error("xmi_gpu_build_surrogate failed");
    xmi_surrogate_free(sg);
    return 0;
  }
  sg->report[4] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  sg->report[5] = ncell;
  xmi_surrogate_free(in->surrogate);
  in->surrogate = sg;
  if (report)
    for (int k = 0; k < 6; k++) report[k] = sg->report[k];
  return 1;
}

/* The solid angle at (r, theta) depends on the detector radius and the
 * collimator alone, so a network trained for one input serves every input
 * with the same detector; their points outside its checked box go to the
 * integrator. */
int xmi_gpu_share_surrogate(xmi_inputFPtr from, xmi_inputFPtr to) {
  if (!from || !to || !from->surrogate || !to->initialized) {
    xmi_set_error("xmi_gpu_share_surrogate: the source input has no trained surrogate");
    return 0;
  }
  SurrogateState *sg = (SurrogateState *)from->surrogate;
  const xmi::SaGeom g{to->det_radius, to->coll_radius, to->coll_height, to->coll_present};
  if (g.det_radius != sg->geom.det_radius || g.coll_present != sg->geom.coll_present ||
      (g.coll_present && (g.coll_radius != sg->geom.coll_radius || g.coll_height != sg->geom.coll_height))) {
    xmi_set_error("xmi_gpu_share_surrogate: detector or collimator differ from the ones the network was trained for");
    return 0;
  }
  if (to->surrogate == sg) return 1;
  sg->refs++;
  xmi_surrogate_free(to->surrogate);
  to->surrogate = sg;
  return 1;
}

int xmi_surrogate_apply(const void *p, int precision, const void *dev_bundles, int n_cfg, void *events,
                        const unsigned long long *count, long long cap, unsigned long long *fallbacks, int *fb_list,
                        unsigned long long *fb_count, int *err, void *stream) {
  using namespace xmi::mlp;
  const SurrogateState *sg = (const SurrogateState *)p;
  if (!sg) return 0;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == 0) {
    cudaFuncSetAttribute(omega_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    omega_kernel<double><<<sms, kFwdThreads, SM_TOTAL, st>>>(sg->packed_d, sg->theta_d, sg->dom, sg->flags_d,
                                                      (const xmi::DevBundle<double> *)dev_bundles, n_cfg,
                                                      (xmi::VrEvent<double> *)events, count, cap, fallbacks, fb_list,
                                                      fb_count, sg->patch_of_d, sg->patches_d, err);
    omega_fallback_kernel<double><<<sms * 8, 256, 0, st>>>((const xmi::DevBundle<double> *)dev_bundles, n_cfg,
                                                          (xmi::VrEvent<double> *)events, fb_list, fb_count, cap);
  } else {
    cudaFuncSetAttribute(omega_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    omega_kernel<float><<<sms, kFwdThreads, SM_TOTAL, st>>>(sg->packed_d, sg->theta_d, sg->dom, sg->flags_d,
                                                     (const xmi::DevBundle<float> *)dev_bundles, n_cfg,
                                                     (xmi::VrEvent<float> *)events, count, cap, fallbacks, fb_list,
                                                     fb_count, sg->patch_of_d, sg->patches_d, err);
    omega_fallback_kernel<float><<<sms * 8, 256, 0, st>>>((const xmi::DevBundle<float> *)dev_bundles, n_cfg,
                                                         (xmi::VrEvent<float> *)events, fb_list, fb_count, cap);
  }
  return cudaGetLastError() == cudaSuccess ? 1 : 0;
}

int xmi_gpu_surrogate_eval(xmi_inputFPtr in, int n, const double *r, const double *theta, double *omega,
                           int *source) {
  using namespace xmi::mlp;
  if (!in || !in->surrogate || n < 0 || (n > 0 && (!r || !theta || !omega || !source))) {
    xmi_set_error("xmi_gpu_surrogate_eval: no trained surrogate or bad arguments");
    return 0;
  }
  if (n == 0) return 1;
  if (!surrogate_device_ok()) return 0;
  const SurrogateState *sg = (const SurrogateState *)in->surrogate;
  /* where each point is served: decided on the host with the network's own
   * cell map; the network runs on every point (one batched forward) */
  std::vector<float> feat(3 * (size_t)n), pred(n);
  std::vector<int> cell_of(n);
  std::vector<unsigned char> flags(sg->dom.ncr * sg->dom.nct);
  std::vector<int> patch_of(flags.size());
  for (int i = 0; i < n; i++) {
    bool inside;
    features_of(sg->dom, r[i], theta[i], &feat[3 * (size_t)i], inside, cell_of[i]);
    source[i] = !(theta[i] >= (double)sg->dom.tmin) ? 3 : (!inside ? 2 : 0);
  }
  float *feat_d = nullptr, *pred_d = nullptr;
  int *err_d = nullptr;
  bool ok = cudaMalloc(&feat_d, sizeof(float) * 3 * (size_t)n) == cudaSuccess &&
            cudaMalloc(&pred_d, sizeof(float) * (size_t)n) == cudaSuccess &&
            cudaMalloc(&err_d, sizeof(int)) == cudaSuccess;
  std::vector<float> patches;
  if (ok) {
    cudaMemcpy(feat_d, feat.data(), sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemset(err_d, 0, sizeof(int));
    ok = device_forward(*sg, feat_d, pred_d, n, err_d);
    int h_err = 0;
    if (ok) {
      cudaMemcpy(&h_err, err_d, sizeof(int), cudaMemcpyDeviceToHost);
      cudaMemcpy(pred.data(), pred_d, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost);
      cudaMemcpy(flags.data(), sg->flags_d, flags.size(), cudaMemcpyDeviceToHost);
      cudaMemcpy(patch_of.data(), sg->patch_of_d, sizeof(int) * patch_of.size(), cudaMemcpyDeviceToHost);
      patches.resize((size_t)(sg->n_patch > 0 ? sg->n_patch : 1) * kPatchNodes);
      if (sg->n_patch > 0)
        cudaMemcpy(patches.data(), sg->patches_d, sizeof(float) * (size_t)sg->n_patch * kPatchNodes,
                   cudaMemcpyDeviceToHost);
      ok = cudaGetLastError() == cudaSuccess;
    }
    if (h_err) {
      xmi_set_error("xmi_gpu_surrogate_eval: tensor-core wait ran out");
      ok = false;
    }
  }
  cudaFree(feat_d);
  cudaFree(pred_d);
  cudaFree(err_d);
  if (!ok) {
    if (!*xmi_gpu_last_error()) xmi_set_error("xmi_gpu_surrogate_eval: CUDA error");
    return 0;
  }
  /* the same choices as omega_kernel (the host exponential in place of the
   * device's fast one: they differ by about 1e-6 relative) */
  for (int i = 0; i < n; i++) {
    if (source[i] == 3) {
      omega[i] = 0.0;
    } else if (source[i] == 2) {
      omega[i] = -1.0;
    } else if (flags[cell_of[i]]) {
      const int pc = patch_of[cell_of[i]];
      if (pc >= 0) {
        source[i] = 1;
        omega[i] = patch_omega(sg->dom, patches.data() + (size_t)pc * kPatchNodes, logf((float)r[i]),
                               (float)theta[i], cell_of[i]);
      } else {
        source[i] = 2;
        omega[i] = -1.0;
      }
    } else {
      const float o = expf(pred[i]) - sg->dom.eps;
      omega[i] = o > 0.0f ? o : 0.0f;
    }
  }
  return 1;
}

int xmi_gpu_solid_angle_points(xmi_inputFPtr in, int n, const double *r, const double *theta, int hits,
                               int precision, unsigned long long seed, double *omega) {
  if (!in || !in->initialized || n < 0 || hits < 1 || (n > 0 && (!r || !theta || !omega))) {
    xmi_set_error("xmi_gpu_solid_angle_points: bad arguments");
    return 0;
  }
  if (n == 0) return 1;
  if (!surrogate_device_ok()) return 0;
  const xmi::SaGeom geom{in->det_radius, in->coll_radius, in->coll_height, in->coll_present};
  double *r_d = nullptr, *t_d = nullptr, *o_d = nullptr;
  bool ok = cudaMalloc(&r_d, sizeof(double) * (size_t)n) == cudaSuccess &&
            cudaMalloc(&t_d, sizeof(double) * (size_t)n) == cudaSuccess &&
            cudaMalloc(&o_d, sizeof(double) * (size_t)n) == cudaSuccess;
  if (ok) {
    cudaMemcpy(r_d, r, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(t_d, theta, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (precision == 0)
      xmi::solid_angle_points_kernel<double><<<sms * 8, 256>>>(geom, r_d, t_d, n, hits, seed, o_d);
    else
      xmi::solid_angle_points_kernel<float><<<sms * 8, 256>>>(geom, r_d, t_d, n, hits, seed, o_d);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
         cudaMemcpy(omega, o_d, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(r_d);
  cudaFree(t_d);
  cudaFree(o_d);
  if (!ok) xmi_set_error("xmi_gpu_solid_angle_points: CUDA error");
  return ok ? 1 : 0;
}

int xmi_solid_angle_deferred(int precision, const void *dev_bundles, int n_cfg, void *events,
                             const unsigned long long *count, long long cap, int *fb_list,
                             unsigned long long *fb_count, void *stream) {
  using namespace xmi::mlp;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == 0) {
    collect_pending_kernel<double><<<sms * 4, 256, 0, st>>>((const xmi::VrEvent<double> *)events, count, cap, fb_list,
                                                           fb_count);
    omega_fallback_kernel<double><<<sms * 8, 256, 0, st>>>((const xmi::DevBundle<double> *)dev_bundles, n_cfg,
                                                          (xmi::VrEvent<double> *)events, fb_list, fb_count, cap);
  } else {
    collect_pending_kernel<float><<<sms * 4, 256, 0, st>>>((const xmi::VrEvent<float> *)events, count, cap, fb_list,
                                                          fb_count);
    omega_fallback_kernel<float><<<sms * 8, 256, 0, st>>>((const xmi::DevBundle<float> *)dev_bundles, n_cfg,
                                                         (xmi::VrEvent<float> *)events, fb_list, fb_count, cap);
  }
  return cudaGetLastError() == cudaSuccess ? 1 : 0;
}

int xmi_gpu_surrogate_report(xmi_inputFPtr in, double *report) {
  if (!in || !in->surrogate || !report) return 0;
  const SurrogateState *sg = (const SurrogateState *)in->surrogate;
  for (int k = 0; k < 6; k++) report[k] = sg->report[k];
  return 1;
}
}
