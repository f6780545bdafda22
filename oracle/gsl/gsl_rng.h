/*
 * Stand-in for the part of GSL's <gsl/gsl_rng.h> that the reference uses, so
 * that the reference's own, unmodified sources compile here as the oracle
 * (GSL itself is neither installed nor vendored with the reference).
 * TEST INFRASTRUCTURE ONLY.
 *
 * Used by the reference: gsl_rng_alloc(gsl_rng_mt19937), gsl_rng_set,
 * gsl_rng_uniform, gsl_rng_free (v25/classes.hpp:155-176, v25/main.cpp:209-211,
 * v25/functions.cpp:2956), gsl_rng_fwrite / gsl_rng_fread
 * (v25/classes.cpp:353,364).  The saved state is written as GSL lays out
 * its MT19937 state on LP64 (624 unsigned longs, then an int, padded), so
 * the files have the same 5000-byte size as the reference's ran_state*.dat.
 */
#ifndef MDSC_GSL_RNG_SHIM_H
#define MDSC_GSL_RNG_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include "../mt19937.h"

typedef struct {
  const char* name;
} gsl_rng_type;

typedef struct {
  const gsl_rng_type* type;
  mdsc_mt19937 state;
} gsl_rng;

static const gsl_rng_type mdsc_gsl_mt19937_type = {"mt19937"};
static const gsl_rng_type* const gsl_rng_mt19937 = &mdsc_gsl_mt19937_type;

static inline gsl_rng* gsl_rng_alloc(const gsl_rng_type* T) {
  gsl_rng* r = (gsl_rng*)malloc(sizeof(gsl_rng));
  r->type = T;
  mdsc_mt_seed(&r->state, 0); /* GSL seeds new generators with its default seed */
  return r;
}

static inline void gsl_rng_set(const gsl_rng* r, unsigned long seed) {
  mdsc_mt_seed(&((gsl_rng*)r)->state, seed);
}

static inline double gsl_rng_uniform(const gsl_rng* r) {
  return mdsc_mt_uniform(&((gsl_rng*)r)->state);
}

static inline void gsl_rng_free(gsl_rng* r) { free(r); }

typedef struct {
  unsigned long mt[MDSC_MT_N];
  int mti;
} mdsc_gsl_mt_file_state;

static inline int gsl_rng_fwrite(FILE* stream, const gsl_rng* r) {
  mdsc_gsl_mt_file_state s;
  for (int i = 0; i < MDSC_MT_N; ++i) s.mt[i] = r->state.mt[i];
  s.mti = r->state.mti;
  return fwrite(&s, sizeof(s), 1, stream) == 1 ? 0 : 1;
}

static inline int gsl_rng_fread(FILE* stream, gsl_rng* r) {
  mdsc_gsl_mt_file_state s;
  if (fread(&s, sizeof(s), 1, stream) != 1) return 1;
  for (int i = 0; i < MDSC_MT_N; ++i) r->state.mt[i] = (uint32_t)s.mt[i];
  r->state.mti = s.mti;
  return 0;
}

#endif
