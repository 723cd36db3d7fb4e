/*
 * hlbl_gb300_rng.h -- counter-based propagator fixtures (host and device).
 *
 * Two generators, both keyed by (seed, global site, flavour, source
 * spin-colour, component) so that every value depends only on the seed and
 * the global site, never on the process grid or the thread that makes it:
 *
 *  - hlbl_rng_uniform_entry: the reference's RandomProvider fixture, uniform
 *    in [-1, 1) from a splitmix64 finaliser (src/provider.cpp:10-21, key and
 *    global-site hash at :36-49, per-source seed folding at :59-64). All of it
 *    is integer arithmetic plus exact power-of-two scaling, so it is
 *    bit-identical on every platform.
 *  - hlbl_rng_gaussian_entry: i.i.d. complex Gaussian entries, mean 0 and
 *    E|z|^2 = 1 (each real part N(0, 1/2)), by Box-Muller on two uniforms
 *    drawn from the same key scheme. log/cos/sin are not exactly rounded, so
 *    host and device values may differ in the last bits; tests that compare
 *    a GPU result with the oracle copy one side's block to the other.
 */
#ifndef HLBL_GB300_RNG_H
#define HLBL_GB300_RNG_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define HLBL_RNG_HD __host__ __device__ __forceinline__
#else
#define HLBL_RNG_HD static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

HLBL_RNG_HD uint64_t hlbl_rng_hash64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

/* Global-site key of (t, x, y, z). */
HLBL_RNG_HD uint64_t hlbl_rng_site_key(int t, int x, int y, int z) {
  return (((uint64_t)t * 1000003u + (uint64_t)x) * 1000003u + (uint64_t)y) *
             1000003u + (uint64_t)z;
}

/* One source position's seed, folded from a run seed and its global site. */
HLBL_RNG_HD uint64_t hlbl_rng_source_seed(uint64_t seed, const int gsx[4]) {
  for (int i = 0; i < 4; ++i) seed = hlbl_rng_hash64(seed ^ (uint64_t)(gsx[i] + 1));
  return seed;
}

/* Reference fixture: real component c (0..23) of block row (f, ia) at the
 * global site with key g. Uniform in [-1, 1). */
HLBL_RNG_HD double hlbl_rng_uniform_entry(uint64_t seed, uint64_t g, int f, int ia,
                                          int c) {
  uint64_t const key = ((g * 2 + (uint64_t)f) * 12 + (uint64_t)ia) * 24 + (uint64_t)c +
                       seed * 0x2545F4914F6CDD1DULL;
  return (double)(hlbl_rng_hash64(key) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

/* Gaussian fixture: complex component c (0..11) of block row (f, ia). */
HLBL_RNG_HD void hlbl_rng_gaussian_entry(uint64_t seed, uint64_t g, int f, int ia, int c,
                                         double* re, double* im) {
  uint64_t const key = ((g * 2 + (uint64_t)f) * 12 + (uint64_t)ia) * 12 + (uint64_t)c +
                       seed * 0x2545F4914F6CDD1DULL + 0x5851F42D4C957F2DULL;
  uint64_t const h1 = hlbl_rng_hash64(key);
  uint64_t const h2 = hlbl_rng_hash64(h1);
  double const u1 = (double)((h1 >> 11) + 1) * (1.0 / 9007199254740992.0); /* (0,1] */
  double const u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);      /* [0,1) */
  double const r = sqrt(-log(u1));
  double const a = 6.283185307179586476925286766559 * u2;
  *re = r * cos(a);
  *im = r * sin(a);
}

#ifdef __cplusplus
}
#endif

#endif /* HLBL_GB300_RNG_H */
