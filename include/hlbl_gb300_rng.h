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
 *    drawn from the same key scheme. The logarithm and the sine and cosine
 *    are this header's own (hlbl_rng_log, hlbl_rng_sincos_turns): exact
 *    reductions (frexp, scaling by powers of two, floor) and fixed
 *    polynomials built only from IEEE-rounded multiplies, adds, fused
 *    multiply-adds and one division, written so that no compiler may fuse
 *    or reorder them (device: __dmul_rn, __dadd_rn, __fma_rn; host: plain
 *    operators, compiled without contraction) -- so host and device
 *    produce the same bits.
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

/* Arithmetic that no compiler fuses or reorders: on the device the
 * round-to-nearest intrinsics; on the host the operators (host code that
 * includes this header is compiled with -ffp-contract=off, or in a strict ISO
 * C mode where that is the default). */
#if defined(__CUDA_ARCH__)
#define HLBL_RNG_MUL(a, b) __dmul_rn((a), (b))
#define HLBL_RNG_ADD(a, b) __dadd_rn((a), (b))
#define HLBL_RNG_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
#define HLBL_RNG_MUL(a, b) ((a) * (b))
#define HLBL_RNG_ADD(a, b) ((a) + (b))
#define HLBL_RNG_FMA(a, b, c) fma((a), (b), (c))
#endif

/* log(x) for x in (0, 1]: x = m 2^e with m in [sqrt(1/2), sqrt(2)) (exact),
 * log m = 2 atanh(s) = 2 s (1 + s^2/3 + s^4/5 + ...), s = (m - 1)/(m + 1),
 * |s| <= 0.1716, the series to s^22 (the next term is below 1e-18 of the
 * sum), and e log 2 with log 2 split into a head exact in e * head and a tail. */
HLBL_RNG_HD double hlbl_rng_log(double x) {
  int e = 0;
  double m = frexp(x, &e); /* x = m 2^e, m in [1/2, 1) */
  if (m < 0.70710678118654752440) {
    m = HLBL_RNG_MUL(m, 2.0);
    e -= 1;
  }
  double const s = HLBL_RNG_ADD(m, -1.0) / HLBL_RNG_ADD(m, 1.0);
  double const z = HLBL_RNG_MUL(s, s);
  double p = 1.0 / 23.0;
  p = HLBL_RNG_FMA(p, z, 1.0 / 21.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 19.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 17.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 15.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 13.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 11.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 9.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 7.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 5.0);
  p = HLBL_RNG_FMA(p, z, 1.0 / 3.0);
  double const lm = HLBL_RNG_FMA(HLBL_RNG_MUL(2.0 * s, z), p, 2.0 * s); /* 2s + 2s z p */
  double const ed = (double)e;
  /* log 2 = 0x1.62e42fefa3800p-1 + 5.497923018708371e-14 (the head has 42
   * significant bits, so e * head is exact for |e| < 2048) */
  return HLBL_RNG_ADD(HLBL_RNG_MUL(ed, 6.93147180559890330187e-01),
                      HLBL_RNG_FMA(ed, 5.497923018708371e-14, lm));
}

/* cos(2 pi t) and sin(2 pi t) for t in [0, 1): octant k = floor(8 t) and its
 * fraction f are exact; the angle within [0, pi/4] is th = g pi/4 with g = f
 * (k even) or 1 - f (k odd, exact), and cos th, sin th are their Taylor
 * polynomials (to th^20 and th^19: the next terms are below 2e-18); the
 * octant's symmetry then maps them to the full angle. */
HLBL_RNG_HD void hlbl_rng_sincos_turns(double t, double* c, double* s) {
  double const t8 = HLBL_RNG_MUL(t, 8.0);
  double const kf = floor(t8);
  int const k = (int)kf;
  double const f = HLBL_RNG_ADD(t8, -kf);
  double const g = (k & 1) ? HLBL_RNG_ADD(1.0, -f) : f;
  double const th = HLBL_RNG_MUL(g, 0.78539816339744830962);
  double const z = HLBL_RNG_MUL(th, th);
  /* sin th = th (1 - z/3! + z^2/5! - ...), cos th = 1 - z/2! + z^2/4! - ... */
  double ps = -1.0 / 121645100408832000.0;          /* -1/19! */
  ps = HLBL_RNG_FMA(ps, z, 1.0 / 355687428096000.0); /* 1/17! */
  ps = HLBL_RNG_FMA(ps, z, -1.0 / 1307674368000.0);  /* -1/15! */
  ps = HLBL_RNG_FMA(ps, z, 1.0 / 6227020800.0);      /* 1/13! */
  ps = HLBL_RNG_FMA(ps, z, -1.0 / 39916800.0);       /* -1/11! */
  ps = HLBL_RNG_FMA(ps, z, 1.0 / 362880.0);          /* 1/9! */
  ps = HLBL_RNG_FMA(ps, z, -1.0 / 5040.0);           /* -1/7! */
  ps = HLBL_RNG_FMA(ps, z, 1.0 / 120.0);             /* 1/5! */
  ps = HLBL_RNG_FMA(ps, z, -1.0 / 6.0);              /* -1/3! */
  double const sn = HLBL_RNG_FMA(HLBL_RNG_MUL(th, z), ps, th);
  double pc = 1.0 / 2432902008176640000.0;           /* 1/20! */
  pc = HLBL_RNG_FMA(pc, z, -1.0 / 6402373705728000.0); /* -1/18! */
  pc = HLBL_RNG_FMA(pc, z, 1.0 / 20922789888000.0);  /* 1/16! */
  pc = HLBL_RNG_FMA(pc, z, -1.0 / 87178291200.0);    /* -1/14! */
  pc = HLBL_RNG_FMA(pc, z, 1.0 / 479001600.0);       /* 1/12! */
  pc = HLBL_RNG_FMA(pc, z, -1.0 / 3628800.0);        /* -1/10! */
  pc = HLBL_RNG_FMA(pc, z, 1.0 / 40320.0);           /* 1/8! */
  pc = HLBL_RNG_FMA(pc, z, -1.0 / 720.0);            /* -1/6! */
  pc = HLBL_RNG_FMA(pc, z, 1.0 / 24.0);              /* 1/4! */
  pc = HLBL_RNG_FMA(pc, z, -0.5);                    /* -1/2! */
  double const cs = HLBL_RNG_FMA(z, pc, 1.0);
  switch (k) {
    case 0: *c = cs; *s = sn; break;
    case 1: *c = sn; *s = cs; break;
    case 2: *c = -sn; *s = cs; break;
    case 3: *c = -cs; *s = sn; break;
    case 4: *c = -cs; *s = -sn; break;
    case 5: *c = -sn; *s = -cs; break;
    case 6: *c = sn; *s = -cs; break;
    default: *c = cs; *s = -sn; break;
  }
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
  double const r = sqrt(-hlbl_rng_log(u1));
  double cs, sn;
  hlbl_rng_sincos_turns(u2, &cs, &sn);
  *re = HLBL_RNG_MUL(r, cs);
  *im = HLBL_RNG_MUL(r, sn);
}

#ifdef __cplusplus
}
#endif

#endif /* HLBL_GB300_RNG_H */
