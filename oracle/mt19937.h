/*
 * MT19937 Mersenne Twister (Matsumoto & Nishimura, ACM TOMACS 8(1), 1998),
 * written from the published algorithm.  TEST INFRASTRUCTURE ONLY: used by
 * the CPU oracle (the checker) and by the gsl_rng stand-in that lets the
 * unmodified reference compile; the GPU product never links it.
 *
 * The reference draws every random number through GSL's `gsl_rng_mt19937`
 * (v25/classes.hpp:150-181, v25/main.cpp:209-211).  GSL's generator is the
 * 2002 `init_genrand` seeding of MT19937 with seed 0 mapped to 4357, and
 * `gsl_rng_uniform` returns the 32-bit output divided by 2^32.  Those three
 * facts are what this file reproduces.
 */
#ifndef MDSC_ORACLE_MT19937_H
#define MDSC_ORACLE_MT19937_H

#include <stdint.h>

#define MDSC_MT_N 624
#define MDSC_MT_M 397

typedef struct {
  uint32_t mt[MDSC_MT_N];
  int mti;
} mdsc_mt19937;

static inline void mdsc_mt_seed(mdsc_mt19937* g, unsigned long seed) {
  uint32_t s = (uint32_t)(seed & 0xffffffffUL);
  if (s == 0) s = 4357u; /* GSL maps seed 0 to 4357 */
  g->mt[0] = s;
  for (int i = 1; i < MDSC_MT_N; ++i)
    g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  g->mti = MDSC_MT_N;
}

static inline uint32_t mdsc_mt_next(mdsc_mt19937* g) {
  const uint32_t upper = 0x80000000u, lower = 0x7fffffffu, matrix_a = 0x9908b0dfu;
  if (g->mti >= MDSC_MT_N) {
    int k;
    for (k = 0; k < MDSC_MT_N - MDSC_MT_M; ++k) {
      uint32_t y = (g->mt[k] & upper) | (g->mt[k + 1] & lower);
      g->mt[k] = g->mt[k + MDSC_MT_M] ^ (y >> 1) ^ ((y & 1u) ? matrix_a : 0u);
    }
    for (; k < MDSC_MT_N - 1; ++k) {
      uint32_t y = (g->mt[k] & upper) | (g->mt[k + 1] & lower);
      g->mt[k] = g->mt[k + (MDSC_MT_M - MDSC_MT_N)] ^ (y >> 1) ^ ((y & 1u) ? matrix_a : 0u);
    }
    {
      uint32_t y = (g->mt[MDSC_MT_N - 1] & upper) | (g->mt[0] & lower);
      g->mt[MDSC_MT_N - 1] = g->mt[MDSC_MT_M - 1] ^ (y >> 1) ^ ((y & 1u) ? matrix_a : 0u);
    }
    g->mti = 0;
  }
  uint32_t y = g->mt[g->mti++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

/* uniform in [0,1): 32-bit draw / 2^32, as gsl_rng_uniform does for MT19937 */
static inline double mdsc_mt_uniform(mdsc_mt19937* g) {
  return (double)mdsc_mt_next(g) / 4294967296.0;
}

#endif
