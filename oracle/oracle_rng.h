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
#endif
