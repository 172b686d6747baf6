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
 * Forward kernel: one CTA of 128 threads per SM, weights resident in shared
 * memory (packed once per launch), 128 queries per tile.  Thread t owns
 * query row t of the tile: it writes the row's features / activations into
 * the K-major operand tile, and after each layer reads its accumulator row
 * back from tensor memory (TMEM lanes 32 w .. 32 w + 31 belong to warp w).
 * Thread 0 issues the MMAs: layer 0 is one M128 N128 K16 instruction,
 * layers 1-3 eight K16 steps each.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

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

/* shared-memory plan of the forward kernel (offsets in bytes) */
constexpr int SM_W = 0;                           /* packed weights */
constexpr int SM_X0 = SM_W + PACK_BYTES;          /* input tile [128 x 16] */
constexpr int SM_A = SM_X0 + H * KIN * 2;         /* activation tile [128 x 128] */
constexpr int SM_BIAS = SM_A + H * H * 2;         /* b0..b3 FP32 */
constexpr int SM_WO = SM_BIAS + 4 * H * 4;        /* w_o FP32 */
constexpr int SM_BAR = SM_WO + H * 4;             /* mbarrier, TMEM address */
constexpr int SM_TOTAL = SM_BAR + 16;

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

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

/* features [n][3] (already scaled) -> out [n] = network output (log solid
 * angle); *err set non-zero when a wait ran out */
__global__ void __launch_bounds__(128, 1) forward_kernel(const unsigned char *packed, const float *theta,
                                                         const float *features, float *out, int n, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5;
  uint64_t *mbar = (uint64_t *)(sm + SM_BAR);
  uint32_t *tmem_slot = (uint32_t *)(sm + SM_BAR + 8);
  float *bias = (float *)(sm + SM_BIAS), *wo = (float *)(sm + SM_WO);

  /* weights and biases into shared memory */
  for (int i = tid; i < PACK_BYTES / 16; i += blockDim.x) ((uint4 *)(sm + SM_W))[i] = ((const uint4 *)packed)[i];
  for (int i = tid; i < H; i += blockDim.x) {
    bias[i] = theta[OFF_B0 + i];
    for (int l = 1; l <= 3; l++) bias[l * H + i] = theta[off_b(l) + i];
    wo[i] = theta[OFF_WO + i];
  }
  for (int i = tid; i < H * KIN * 2 / 16; i += blockDim.x) ((uint4 *)(sm + SM_X0))[i] = make_uint4(0, 0, 0, 0);
  const float bo = theta[OFF_BO];
  if (warp == 0) umma::tmem_alloc(tmem_slot, 128);
  if (tid == 0) {
    umma::mbar_init(mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_proxy_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  const uint32_t idesc = umma::idesc_bf16_f32(128, 128);
  const uint32_t s_x0 = umma::smem_u32(sm + SM_X0), s_a = umma::smem_u32(sm + SM_A), s_w = umma::smem_u32(sm + SM_W);
  uint32_t phase = 0;
  bool failed = false;

  for (int tile = blockIdx.x; tile * 128 < n && !failed; tile += gridDim.x) {
    const int row = tile * 128 + tid;
    const bool valid = row < n;
#pragma unroll
    for (int k = 0; k < NIN; k++) {
      const float v = valid ? features[(size_t)row * NIN + k] : 0.0f;
      *(__nv_bfloat16 *)(sm + SM_X0 + umma::kmajor_offset(tid, k, KIN)) = __float2bfloat16_rn(v);
    }
    float acc_out = bo;
    for (int l = 0; l < 4; l++) {
      umma::fence_proxy_async_smem();
      umma::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        umma::fence_after_sync();
        if (l == 0) {
          umma::mma_bf16(tmem, umma::smem_desc(s_x0, 128, 256), umma::smem_desc(s_w, 128, 256), idesc, false);
        } else {
          const uint32_t wl = s_w + W0_BYTES + (l - 1) * WL_BYTES;
#pragma unroll
          for (int kk = 0; kk < H / 16; kk++)
            umma::mma_bf16(tmem, umma::smem_desc(s_a + kk * 256, 128, 2048), umma::smem_desc(wl + kk * 256, 128, 2048),
                           idesc, kk > 0);
        }
        umma::mma_commit(mbar);
      }
      const bool ok = umma::mbar_wait(mbar, phase);
      phase ^= 1u;
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      umma::fence_after_sync();
      /* epilogue of layer l: bias, SiLU; the next layer's operand or the output */
#pragma unroll 1
      for (int c = 0; c < H / 32; c++) {
        float v[32];
        umma::tmem_ld_32x32b_x32(trow + c * 32, v);
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const float h = silu(v[j] + bias[l * H + c * 32 + j]);
          if (l < 3)
            *(__nv_bfloat16 *)(sm + SM_A + umma::kmajor_offset(tid, c * 32 + j, H)) = __float2bfloat16_rn(h);
          else
            acc_out += h * wo[c * 32 + j];
        }
      }
    }
    if (!failed && valid) out[row] = acc_out;
  }
  if (failed && tid == 0) atomicExch(err, 1);
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 128);
}

}  // namespace mlp
}  // namespace xmi

extern "C" {

int xmi_mlp_nparam(void) { return xmi::mlp::NPARAM; }

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
    forward_kernel<<<tiles < sms ? tiles : sms, 128, SM_TOTAL>>>(d_pack, d_theta, d_feat, d_out, n, d_err);
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
}
