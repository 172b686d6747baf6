/*
 * TEST INFRASTRUCTURE (oracle) -- not part of the engine.
 *
 * Philox4x32-10 (Salmon et al., SC'11) and the engine's stream convention:
 * key = 64-bit seed, counter = (block, stream, id_lo, id_hi), two 53-bit
 * uniforms per block.  Written independently of the engine so that the
 * known-answer test of tests/test_oracle.py checks both against the
 * published vectors.
 */
#ifndef XMIMSIM_ORACLE_RNG_H
#define XMIMSIM_ORACLE_RNG_H
#include <stdint.h>

typedef struct {
  uint32_t key[2];
  uint32_t ctr[4];
  uint32_t out[4];
  int used;
} orng;

static inline void orng_block(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  int r;
  for (r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline void orng_init(orng *g, uint64_t seed, uint64_t id, uint32_t stream) {
  g->key[0] = (uint32_t)seed;
  g->key[1] = (uint32_t)(seed >> 32);
  g->ctr[0] = 0;
  g->ctr[1] = stream;
  g->ctr[2] = (uint32_t)id;
  g->ctr[3] = (uint32_t)(id >> 32);
  g->used = 2;
}

static inline double orng_uniform(orng *g) {
  uint32_t a, b;
  if (g->used == 2) {
    orng_block(g->ctr, g->key, g->out);
    g->ctr[0] += 1;
    g->used = 0;
  }
  a = g->out[2 * g->used];
  b = g->out[2 * g->used + 1];
  g->used++;
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) / 9007199254740992.0;
}

/* Threefry4x32-20 (Salmon et al., SC'11), the generator of the reference's
 * OpenCL solid-angle kernel (src/xmi_kernels.cl through Random123), written
 * from the published description: Threefish-style add/rotate/xor rounds on
 * word pairs (0,1),(2,3) in even rounds and (0,3),(2,1) in odd rounds, a key
 * injection after every fourth round, Skein parity word 0x1BD11BDA. */
static inline uint32_t orot32(uint32_t x, unsigned n) { return (x << n) | (x >> (32u - n)); }

static inline void othreefry4x32(const uint32_t in[4], const uint32_t key[4], uint32_t out[4]) {
  static const unsigned rot_a[8] = {10, 11, 13, 23, 6, 17, 25, 18};
  static const unsigned rot_b[8] = {26, 21, 27, 5, 20, 11, 10, 20};
  uint32_t ks[5], x[4];
  int round, i;
  ks[4] = 0x1BD11BDAu;
  for (i = 0; i < 4; i++) {
    ks[i] = key[i];
    ks[4] ^= key[i];
    x[i] = in[i] + key[i];
  }
  for (round = 0; round < 20; round++) {
    const int a = (round & 1) ? 3 : 1, c = (round & 1) ? 1 : 3;
    x[0] += x[a];
    x[a] = orot32(x[a], rot_a[round & 7]) ^ x[0];
    x[2] += x[c];
    x[c] = orot32(x[c], rot_b[round & 7]) ^ x[2];
    if ((round & 3) == 3) {
      const unsigned s = (unsigned)(round + 1) / 4u;
      for (i = 0; i < 4; i++) x[i] += ks[(s + (unsigned)i) % 5u];
      x[3] += s;
    }
  }
  for (i = 0; i < 4; i++) out[i] = x[i];
}

/* the OpenCL kernel's per-point stream (src/xmi_kernels.cl:226-227,393-404):
 * key (r index, 0xdecafbad, 0xfacebead, theta index), counter
 * (j, 0xf00dcafe, 0xdeadbeef, 0xbeeff00d), j incremented before each block;
 * the four words of a block are consumed in order as float(word) / 2^32 */
typedef struct {
  uint32_t key[4], ctr[4], out[4];
  int used;
} oclrng;

static inline void oclrng_init(oclrng *g, uint32_t ir, uint32_t it) {
  g->key[0] = ir; g->key[1] = 0xdecafbadu; g->key[2] = 0xfacebeadu; g->key[3] = it;
  g->ctr[0] = 0u; g->ctr[1] = 0xf00dcafeu; g->ctr[2] = 0xdeadbeefu; g->ctr[3] = 0xbeeff00du;
  g->used = 4;
}

static inline double oclrng_uniform(oclrng *g) {
  float u;
  if (g->used == 4) {
    g->ctr[0] += 1u;
    othreefry4x32(g->ctr, g->key, g->out);
    g->used = 0;
  }
  u = (float)g->out[g->used++] / 4294967296.0f;
  return (double)u;
}
#endif
