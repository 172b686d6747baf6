/*
 * Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11), written from the
 * published round function.  Used host- and device-side.
 *
 * Stream layout of the engine: key = 64-bit seed; counter =
 *   (block, stream, id_lo, id_hi)
 * where `id` is the photon (or grid point) and `stream` names the phase of
 * that photon (0 = source sampling, k = the step leading to interaction k,
 * 0x80000000|k = off-grid solid-angle integral of interaction k,
 * 0xF0000000 = solid-angle grid point).  Every block yields two uniform
 * doubles of 53 bits, consumed in order, so a photon's draw sequence is a
 * pure function of (seed, photon, phase) and identical on CPU and GPU.
 */
#ifndef XMIMSIM_GB300_PHILOX_H
#define XMIMSIM_GB300_PHILOX_H

#include <stdint.h>

#ifdef __CUDACC__
#define XMI_HD __host__ __device__ __forceinline__
#else
#define XMI_HD static inline
#endif

#define XMI_PHILOX_M0 0xD2511F53u
#define XMI_PHILOX_M1 0xCD9E8D57u
#define XMI_PHILOX_W0 0x9E3779B9u
#define XMI_PHILOX_W1 0xBB67AE85u

typedef struct {
  uint32_t v[4];
} xmi_u32x4;

XMI_HD void xmi_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
#ifdef __CUDA_ARCH__
  *hi = __umulhi(a, b);
  *lo = a * b;
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
#endif
}

XMI_HD xmi_u32x4 xmi_philox4x32_10(xmi_u32x4 c, uint32_t k0, uint32_t k1) {
  int r;
  for (r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    xmi_u32x4 n;
    if (r > 0) {
      k0 += XMI_PHILOX_W0;
      k1 += XMI_PHILOX_W1;
    }
    xmi_mulhilo32(XMI_PHILOX_M0, c.v[0], &hi0, &lo0);
    xmi_mulhilo32(XMI_PHILOX_M1, c.v[2], &hi1, &lo1);
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
  }
  return c;
}

typedef struct {
  uint32_t k0, k1;
  xmi_u32x4 ctr;
  xmi_u32x4 buf;
  int pos; /* 0: buf holds two fresh doubles, 1: one left, 2: empty */
} xmi_rng;

XMI_HD void xmi_rng_init(xmi_rng *g, uint64_t seed, uint64_t id, uint32_t stream) {
  g->k0 = (uint32_t)seed;
  g->k1 = (uint32_t)(seed >> 32);
  g->ctr.v[0] = 0u;
  g->ctr.v[1] = stream;
  g->ctr.v[2] = (uint32_t)id;
  g->ctr.v[3] = (uint32_t)(id >> 32);
  g->pos = 2;
}

/* restarts a stream at a saved position: next block counter ctr0 and the
 * number of draws already taken from the block before it (pos, 2 = none left) */
XMI_HD void xmi_rng_resume(xmi_rng *g, uint64_t seed, uint64_t id, uint32_t stream, uint32_t ctr0, int pos) {
  xmi_rng_init(g, seed, id, stream);
  if (pos < 2) {
    g->ctr.v[0] = ctr0 - 1u;
    g->buf = xmi_philox4x32_10(g->ctr, g->k0, g->k1);
  }
  g->ctr.v[0] = ctr0;
  g->pos = pos;
}

/* consumes one draw (two words) and returns its first word: the 32 most
 * significant of the 53 random bits of the uniform xmi_rng_uniform would
 * have returned */
XMI_HD uint32_t xmi_rng_word(xmi_rng *g) {
  uint32_t a;
  if (g->pos >= 2) {
    g->buf = xmi_philox4x32_10(g->ctr, g->k0, g->k1);
    g->ctr.v[0]++;
    g->pos = 0;
  }
  a = g->buf.v[2 * g->pos];
  g->pos++;
  return a;
}

/* uniform double in [0, 1) with 53 random bits */
XMI_HD double xmi_rng_uniform(xmi_rng *g) {
  uint32_t a, b;
  if (g->pos >= 2) {
    g->buf = xmi_philox4x32_10(g->ctr, g->k0, g->k1);
    g->ctr.v[0]++;
    g->pos = 0;
  }
  a = g->buf.v[2 * g->pos];
  b = g->buf.v[2 * g->pos + 1];
  g->pos++;
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* Threefry4x32-20 (Salmon et al., SC'11; the Threefish-style ARX round with
 * the 4x32 rotation schedule of that paper and the Skein key-schedule parity
 * 0x1BD11BDA), written from the published description.  The engine uses it
 * only for the reference solid-angle stream of the OpenCL backend
 * (src/xmi_kernels.cl:219-453): key (r index, 0xdecafbad, 0xfacebead,
 * theta index), counter (j, 0xf00dcafe, 0xdeadbeef, 0xbeeff00d) for the
 * j-th pair of cone samples (j = 1, 2, ...). */
XMI_HD uint32_t xmi_rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

XMI_HD xmi_u32x4 xmi_threefry4x32_20(xmi_u32x4 c, xmi_u32x4 k) {
  const int rot[8][2] = {{10, 26}, {11, 21}, {13, 27}, {23, 5}, {6, 20}, {17, 11}, {25, 10}, {18, 20}};
  uint32_t ks[5];
  uint32_t x0, x1, x2, x3;
  int r;
  ks[4] = 0x1BD11BDAu;
  for (r = 0; r < 4; r++) {
    ks[r] = k.v[r];
    ks[4] ^= k.v[r];
  }
  x0 = c.v[0] + ks[0];
  x1 = c.v[1] + ks[1];
  x2 = c.v[2] + ks[2];
  x3 = c.v[3] + ks[3];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (r = 0; r < 20; r++) {
    if ((r & 1) == 0) {
      x0 += x1; x1 = xmi_rotl32(x1, rot[r & 7][0]); x1 ^= x0;
      x2 += x3; x3 = xmi_rotl32(x3, rot[r & 7][1]); x3 ^= x2;
    } else {
      x0 += x3; x3 = xmi_rotl32(x3, rot[r & 7][0]); x3 ^= x0;
      x2 += x1; x1 = xmi_rotl32(x1, rot[r & 7][1]); x1 ^= x2;
    }
    if ((r & 3) == 3) {
      const uint32_t inj = (uint32_t)((r + 1) >> 2);
      x0 += ks[inj % 5];
      x1 += ks[(inj + 1) % 5];
      x2 += ks[(inj + 2) % 5];
      x3 += ks[(inj + 3) % 5] + inj;
    }
  }
  c.v[0] = x0; c.v[1] = x1; c.v[2] = x2; c.v[3] = x3;
  return c;
}

#endif
