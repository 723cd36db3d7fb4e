/*
 * hlbl_oracle.c -- TEST INFRASTRUCTURE. The CPU oracle for the connected HLbL
 * kernel sum. Only the tests, the smoke check and bench.py's CPU-baseline leg
 * load it, as the checker; the product never calls it.
 *
 * A plain FP64 restatement (OpenMP over sites) of the reference's algorithm:
 *
 *   oracle_dzu_dzsu      pass 1, kernels/cuda_lattice.cu:160-262 (ker_dzu_dzsu)
 *   oracle_insert_gammas host gamma insertion, src/contract.cpp:18-24, 58-77
 *   oracle_4pt           pass 2, kernels/cuda_lattice.cu:277-484
 *                        (ker_4pt_contraction) with the QED calls of :266-275
 *   oracle_kernel_sum    Contractor::kernel_sum, src/contract.cpp:104-114
 *   oracle_fill_*        the block fixtures, src/provider.cpp:25-69
 *
 * and of the 2+2 pieces (kernels/hlbl_kernels/kernels.cu):
 *
 *   oracle_pi            Pi(z)[mu][nu], kernel_pi :241-294
 *   oracle_p1_2p2        P1 slab sums, kernel_p1 :296-339
 *   oracle_p234          P2_0, P2_1, P3, P4_0, P4_1 per target,
 *                        kernel_p20 :374-458, kernel_p21 :461-545,
 *                        kernel_p3 :548-643, kernel_p4 :646-750
 *   oracle_pieces_2p2    compute_2p2_gpu :753-870 with the per-target
 *                        reordering of Contractor::pieces_2p2
 *                        (src/contract.cpp:116-156)
 *
 * The loops follow the reference's order of operations per site; loop
 * invariants are hoisted (gamma-rotated spinors are formed once per site
 * instead of once per inner iteration), which changes no value. Sums over
 * sites use per-thread partials reduced in thread order, so a run is
 * deterministic for a given thread count. The QED kernel is the project's
 * stand-in (include/hlbl_gb300_qed.h), as KQED is not available, or, after
 * oracle_set_qed_dense, the dense test weight of the same header (a tensor
 * with no index structure).
 *
 * Parity pin: these functions are checked against the reference's own
 * sources compiled as a host emulation (oracle/ref_host) through the golden
 * fixtures in tests/golden.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "hlbl_gb300_qed.h"
#include "hlbl_gb300_rng.h"

/* ---- gamma matrices in the cvc basis (src/gamma.cpp:7-45,
 * kernels/cuda_lattice.cu:16-51), as monomial spin matrices:
 * (gamma_g v)[s][c] = i^ph[g][s] * v[src[g][s]][c]. Row 4 is unused. */
static const int g_src[6][4] = {{2, 3, 0, 1}, {3, 2, 1, 0}, {3, 2, 1, 0},
                                {2, 3, 0, 1}, {0, 1, 2, 3}, {0, 1, 2, 3}};
static const int g_ph[6][4] = {{2, 2, 2, 2}, {3, 3, 1, 1}, {2, 0, 0, 2},
                               {3, 1, 1, 3}, {0, 0, 0, 0}, {0, 0, 2, 2}};

/* out = gamma_g in (24 doubles, 12 complex, index 3*spin + colour) */
static void apply_gamma(int g, const double* in, double* out) {
  for (int s = 0; s < 4; ++s) {
    int const j = g_src[g][s], ph = g_ph[g][s];
    for (int c = 0; c < 3; ++c) {
      double const re = in[2 * (3 * j + c)], im = in[2 * (3 * j + c) + 1];
      double* o = out + 2 * (3 * s + c);
      switch (ph) {
        case 0: o[0] = re;  o[1] = im;  break;
        case 1: o[0] = -im; o[1] = re;  break;
        case 2: o[0] = -re; o[1] = -im; break;
        default: o[0] = im; o[1] = -re; break;
      }
    }
  }
}
/* in place: gamma_5 (spins 2 and 3 change sign), cuda_lattice.cu:96-100 */
static void times_g5(double* v) {
  for (int i = 12; i < 24; ++i) v[i] = -v[i];
}

void oracle_apply_gamma(int g, const double* in, double* out) { apply_gamma(g, in, out); }

/* ---- coordinate rules, cuda_lattice.cu:128-154 (VENDORED.md: one rule,
 * [-L/2, L/2), for every QED kernel argument; L/2 -> 0 only for the odd
 * coordinate weights) */
int oracle_coord_map(int xi, int L) { return xi >= L / 2 ? xi - L : xi; }
int oracle_coord_map_zerohalf(int xi, int L) {
  return xi > L / 2 ? xi - L : (xi < L / 2 ? xi : 0);
}
int oracle_mod_pos(int a, int L) {
  int const r = a % L;
  return r < 0 ? r + L : r;
}
int oracle_coord_map_diff(int a, int b, int L) {
  return oracle_coord_map(oracle_mod_pos(a - b, L), L);
}

static int n_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
static int thread_id(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

/* Summation mode. Compensated (the default, used as the checker): every sum
 * over sites, the 144-term corr sums and the 1536-term per-site sum use
 * Neumaier's compensated summation, which removes the order dependence the
 * reference's plain loops have on sums that nearly cancel. Plain: the
 * reference's own plain accumulation, used to time the CPU baseline. */
static int g_compensated = 1;
void oracle_set_compensated(int on) { g_compensated = on != 0; }
int oracle_get_compensated(void) { return g_compensated; }

typedef struct { double s, c; } acc_t;
static inline void acc_add(acc_t* a, double v) {
  if (!g_compensated) { a->s += v; return; }
  double const t = a->s + v;
  a->c += fabs(a->s) >= fabs(v) ? (a->s - t) + v : (v - t) + a->s;
  a->s = t;
}
static inline double acc_get(const acc_t* a) { return a->s + a->c; }

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int oracle_get_threads(void) { return n_threads(); }

/* ---- fixtures (src/provider.cpp) ---- */

/* fill_random_block (provider.cpp:25-57): layout ((f*12+ia)*V + site)*24 + c,
 * site = ((t*LX+x)*LY+y)*LZ+z local, values keyed by the global site. */
void oracle_fill_random_block(const int local[4], const int pc[4], uint64_t seed,
                              double* out) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
#pragma omp parallel for schedule(static)
  for (long long site = 0; site < (long long)V; ++site) {
    int const z = (int)(site % local[3]);
    int const y = (int)((site / local[3]) % local[2]);
    int const x = (int)((site / ((size_t)local[3] * local[2])) % local[1]);
    int const t = (int)(site / ((size_t)local[3] * local[2] * local[1]));
    uint64_t const g = hlbl_rng_site_key(pc[0] * local[0] + t, pc[1] * local[1] + x,
                                         pc[2] * local[2] + y, pc[3] * local[3] + z);
    for (int f = 0; f < 2; ++f)
      for (int ia = 0; ia < 12; ++ia)
        for (int c = 0; c < 24; ++c)
          out[((size_t)(f * 12 + ia) * V + (size_t)site) * 24 + c] =
              hlbl_rng_uniform_entry(seed, g, f, ia, c);
  }
}

/* RandomProvider::compute's per-source seed (provider.cpp:59-64). */
uint64_t oracle_source_seed(uint64_t seed, const int gsx[4]) {
  return hlbl_rng_source_seed(seed, gsx);
}

/* The Gaussian fixture of the benchmark configurations, same layout. */
void oracle_fill_gaussian_block(const int local[4], const int pc[4], uint64_t seed,
                                double* out) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
#pragma omp parallel for schedule(static)
  for (long long site = 0; site < (long long)V; ++site) {
    int const z = (int)(site % local[3]);
    int const y = (int)((site / local[3]) % local[2]);
    int const x = (int)((site / ((size_t)local[3] * local[2])) % local[1]);
    int const t = (int)(site / ((size_t)local[3] * local[2] * local[1]));
    uint64_t const g = hlbl_rng_site_key(pc[0] * local[0] + t, pc[1] * local[1] + x,
                                         pc[2] * local[2] + y, pc[3] * local[3] + z);
    for (int f = 0; f < 2; ++f)
      for (int ia = 0; ia < 12; ++ia)
        for (int c = 0; c < 12; ++c) {
          double* o = out + ((size_t)(f * 12 + ia) * V + (size_t)site) * 24 + 2 * c;
          hlbl_rng_gaussian_entry(seed, g, f, ia, c, o, o + 1);
        }
  }
}

/* ---- the QED kernel (cuda_lattice.cu:266-275 calls QED_Mkernel_L2) ----
 * The stand-in (default) or the dense test weight with a seeded table. */
static double* g_dense = NULL; /* HLBL_QED_DENSE_NB x HLBL_QED_NK, or NULL */

void oracle_set_qed_dense(int on, unsigned long long seed) {
  if (!on) {
    free(g_dense);
    g_dense = NULL;
    return;
  }
  if (!g_dense) g_dense = (double*)malloc(sizeof(double) * HLBL_QED_DENSE_NB * HLBL_QED_NK);
  hlbl_qed_dense_init(g_dense, seed);
}
int oracle_get_qed_dense(void) { return g_dense != NULL; }

static void qed_kernel(const hlbl_qed_params* p, const double x[4], const double y[4],
                       double kerv[6][4][4][4]) {
  if (g_dense) hlbl_qed_dense_kernel(g_dense, x, y, kerv);
  else hlbl_qed_kernel(p, x, y, kerv);
}

void oracle_qed_kernel(double lambda, const double x[4], const double y[4], double* kerv) {
  hlbl_qed_params p;
  hlbl_qed_params_init(&p, lambda);
  qed_kernel(&p, x, y, (double(*)[4][4][4])kerv);
}
void oracle_qed_weights(double lambda, double X, double c, double Y, double* w) {
  hlbl_qed_params p;
  hlbl_qed_params_init(&p, lambda);
  hlbl_qed_weights(&p, X, c, Y, w);
}

static void site_coords(size_t ix, const int local[4], int coord[4]) {
  coord[3] = (int)(ix % local[3]);
  coord[2] = (int)((ix / local[3]) % local[2]);
  coord[1] = (int)((ix / ((size_t)local[3] * local[2])) % local[1]);
  coord[0] = (int)(ix / ((size_t)local[3] * local[2] * local[1]));
}

static const int comb[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

/* ---- pass 1: ker_dzu_dzsu (cuda_lattice.cu:160-262) -------------------
 * dzu[k][ia][ib]  += sum_z conj(fwd_y[1-f][ib](z)) . (z_rho g5 g_sigma - z_sigma g5 g_rho) fwd_src[f][ia](z)
 * dzsu[s][ia][ib] += sum_z conj(fwd_y[1-f][ib](z)) . g5 g_s fwd_src[f][ia](z)
 * z_rho = coord_map_zerohalf((z - gsx)_rho mod L_rho). Adds into dzu, dzsu. */
void oracle_dzu_dzsu(double* dzu, double* dzsu, const double* fwd_src, const double* fwd_y,
                     int iflavor, const int pc[4], const int gsx[4], const int global[4],
                     const int local[4]) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
  int const nt = n_threads();
  acc_t* part = (acc_t*)calloc((size_t)nt * 2880, sizeof(acc_t));
#pragma omp parallel
  {
    acc_t* acc_u = part + (size_t)thread_id() * 2880; /* [6][12][12][2] */
    acc_t* acc_s = acc_u + 1728;                       /* [4][12][12][2] */
#pragma omp for schedule(static)
    for (long long iz = 0; iz < (long long)V; ++iz) {
      int coord[4], zf[4];
      site_coords((size_t)iz, local, coord);
      for (int r = 0; r < 4; ++r) {
        int zr = coord[r] + pc[r] * local[r] - gsx[r];
        zr = (zr + global[r]) % global[r];
        zf[r] = oracle_coord_map_zerohalf(zr, global[r]);
      }
      for (int ia = 0; ia < 12; ++ia) {
        const double* u = fwd_src + ((size_t)(iflavor * 12 + ia) * V + (size_t)iz) * 24;
        double t[4][24]; /* g5 g_s u */
        for (int s = 0; s < 4; ++s) {
          apply_gamma(s, u, t[s]);
          times_g5(t[s]);
        }
        for (int k = 0; k < 6; ++k) {
          int const rho = comb[k][0], sigma = comb[k][1];
          double const fr = zf[rho], fs = zf[sigma];
          for (int ib = 0; ib < 12; ++ib) {
            const double* yb =
                fwd_y + ((size_t)((1 - iflavor) * 12 + ib) * V + (size_t)iz) * 24;
            double re = 0, im = 0;
            for (int i = 0; i < 12; ++i) {
              double const yr = yb[2 * i], yi = yb[2 * i + 1];
              double const sr = t[sigma][2 * i] * fr - t[rho][2 * i] * fs;
              double const si = t[sigma][2 * i + 1] * fr - t[rho][2 * i + 1] * fs;
              re += yr * sr + yi * si;
              im += yr * si - yi * sr;
            }
            acc_add(&acc_u[((k * 12 + ia) * 12 + ib) * 2], re);
            acc_add(&acc_u[((k * 12 + ia) * 12 + ib) * 2 + 1], im);
          }
        }
        for (int s = 0; s < 4; ++s) {
          for (int ib = 0; ib < 12; ++ib) {
            const double* yb =
                fwd_y + ((size_t)((1 - iflavor) * 12 + ib) * V + (size_t)iz) * 24;
            double re = 0, im = 0;
            for (int i = 0; i < 12; ++i) {
              double const yr = yb[2 * i], yi = yb[2 * i + 1];
              re += yr * t[s][2 * i] + yi * t[s][2 * i + 1];
              im += yr * t[s][2 * i + 1] - yi * t[s][2 * i];
            }
            acc_add(&acc_s[((s * 12 + ia) * 12 + ib) * 2], re);
            acc_add(&acc_s[((s * 12 + ia) * 12 + ib) * 2 + 1], im);
          }
        }
      }
    }
  }
  for (int i = 0; i < 2880; ++i) {
    acc_t a = {0.0, 0.0};
    for (int th = 0; th < nt; ++th) {
      acc_add(&a, part[(size_t)th * 2880 + i].s);
      acc_add(&a, part[(size_t)th * 2880 + i].c);
    }
    if (i < 1728) dzu[i] += acc_get(&a);
    else dzsu[i - 1728] += acc_get(&a);
  }
  free(part);
}

/* ---- host glue (contract.cpp:58-77): g_dzu[k][mu][ia] = g_mu g5 dzu[k][ia],
 * g_dzsu[s][mu][ia] = g_mu g5 dzsu[s][ia] (gamma on the 24-vector over ib) */
void oracle_insert_gammas(const double* dzu, const double* dzsu, double* g_dzu,
                          double* g_dzsu) {
  double t[24];
  for (int k = 0; k < 6; ++k)
    for (int ia = 0; ia < 12; ++ia)
      for (int mu = 0; mu < 4; ++mu) {
        memcpy(t, dzu + (k * 12 + ia) * 24, sizeof t);
        times_g5(t);
        apply_gamma(mu, t, g_dzu + ((k * 4 + mu) * 12 + ia) * 24);
      }
  for (int s = 0; s < 4; ++s)
    for (int ia = 0; ia < 12; ++ia)
      for (int mu = 0; mu < 4; ++mu) {
        memcpy(t, dzsu + (s * 12 + ia) * 24, sizeof t);
        times_g5(t);
        apply_gamma(mu, t, g_dzsu + ((s * 4 + mu) * 12 + ia) * 24);
      }
}

/* ---- pass 2: ker_4pt_contraction (cuda_lattice.cu:277-484) ------------
 * Returns the sum over this rank's sites; the caller adds it to its
 * accumulator as the reference's atomicAdd does. */
double oracle_4pt(const double* g_dzu, const double* g_dzsu, const double* fwd_src,
                  const double* fwd_y, int iflavor, const int pc[4], const int gsx[4],
                  double xunit, const int yv[4], double lambda, const int global[4],
                  const int local[4]) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
  int const nt = n_threads();
  acc_t* part = (acc_t*)calloc((size_t)nt, sizeof(acc_t));
  hlbl_qed_params qp;
  hlbl_qed_params_init(&qp, lambda);

  /* ym and the unmapped yv are site-independent (cuda_lattice.cu:411-416) */
  double ym[4];
  for (int r = 0; r < 4; ++r)
    ym[r] = oracle_coord_map(oracle_mod_pos(yv[r], global[r]), global[r]) * xunit;

#pragma omp parallel
  {
    double* corr_I = (double*)malloc(sizeof(double) * 384 * 2);
    double* corr_II = corr_I + 384;
    acc_t sum = {0.0, 0.0};
#pragma omp for schedule(static)
    for (long long ix = 0; ix < (long long)V; ++ix) {
      int coord[4], xv[4], xvzh[4], x_rel[4];
      site_coords((size_t)ix, local, coord);
      for (int r = 0; r < 4; ++r) {
        int xr = coord[r] + pc[r] * local[r] - gsx[r];
        xr = (xr + global[r]) % global[r];
        x_rel[r] = xr;
        xv[r] = oracle_coord_map(xr, global[r]);
        xvzh[r] = oracle_coord_map_zerohalf(xr, global[r]);
      }
      for (int mu = 0; mu < 4; ++mu) {
        /* dxu[ib][ia] = -conj(g5 g_mu fwd_src[1-f][ia]) . fwd_y[f][ib] (:323-345) */
        double dxu[12 * 12 * 2];
        memset(dxu, 0, sizeof dxu);
        for (int ia = 0; ia < 12; ++ia) {
          const double* d = fwd_src + ((size_t)((1 - iflavor) * 12 + ia) * V + (size_t)ix) * 24;
          double t[24];
          apply_gamma(mu, d, t);
          times_g5(t);
          for (int ib = 0; ib < 12; ++ib) {
            const double* u = fwd_y + ((size_t)(iflavor * 12 + ib) * V + (size_t)ix) * 24;
            for (int i = 0; i < 12; ++i) {
              double const tr = t[2 * i], ti = t[2 * i + 1];
              double const ur = u[2 * i], ui = u[2 * i + 1];
              dxu[(ib * 12 + ia) * 2] += -(tr * ur + ti * ui);
              dxu[(ib * 12 + ia) * 2 + 1] += -(tr * ui - ti * ur);
            }
          }
        }
        /* g_dxu[lambda][ia] = g_lambda g5 dxu[ia] (:379-382, hoisted out of k, nu) */
        double g_dxu[4][12][24];
        for (int lam = 0; lam < 4; ++lam)
          for (int ia = 0; ia < 12; ++ia) {
            double t[24];
            apply_gamma(5, dxu + ia * 24, t);
            apply_gamma(lam, t, g_dxu[lam][ia]);
          }
        /* corr_I, corr_II (:346-400) */
        for (int k = 0; k < 6; ++k) {
          int const rho = comb[k][0], sigma = comb[k][1];
          for (int nu = 0; nu < 4; ++nu)
            for (int lam = 0; lam < 4; ++lam) {
              acc_t cI = {0.0, 0.0}, cII = {0.0, 0.0};
              for (int ia = 0; ia < 12; ++ia)
                for (int ib = 0; ib < 12; ++ib) {
                  double const u_re = g_dxu[lam][ia][2 * ib], u_im = g_dxu[lam][ia][2 * ib + 1];
                  double v_re = g_dzu[(((k * 4 + nu) * 12 + ib) * 12 + ia) * 2];
                  double v_im = g_dzu[(((k * 4 + nu) * 12 + ib) * 12 + ia) * 2 + 1];
                  acc_add(&cI, -(u_re * v_re - u_im * v_im));
                  v_re = xvzh[rho] * g_dzsu[(((sigma * 4 + nu) * 12 + ib) * 12 + ia) * 2] -
                         xvzh[sigma] * g_dzsu[(((rho * 4 + nu) * 12 + ib) * 12 + ia) * 2];
                  v_im = xvzh[rho] * g_dzsu[(((sigma * 4 + nu) * 12 + ib) * 12 + ia) * 2 + 1] -
                         xvzh[sigma] * g_dzsu[(((rho * 4 + nu) * 12 + ib) * 12 + ia) * 2 + 1];
                  acc_add(&cII, -(u_re * v_re - u_im * v_im));
                }
              corr_I[((k * 4 + mu) * 4 + nu) * 4 + lam] = acc_get(&cI);
              corr_II[((k * 4 + mu) * 4 + nu) * 4 + lam] = acc_get(&cII);
            }
        }
      }
      /* QED kernel arguments (:403-426) and the three contractions (:428-476) */
      double xm[4], xm_mi_ym[4];
      for (int r = 0; r < 4; ++r) {
        xm[r] = xv[r] * xunit;
        xm_mi_ym[r] = oracle_coord_map_diff(x_rel[r], yv[r], global[r]) * xunit;
      }
      double kerv[6][4][4][4];
      acc_t dtmp = {0.0, 0.0};
      int i;
      qed_kernel(&qp, xm, ym, kerv);
      i = 0;
      for (int k = 0; k < 6; k++)
        for (int mu = 0; mu < 4; mu++)
          for (int nu = 0; nu < 4; nu++)
            for (int lam = 0; lam < 4; lam++) acc_add(&dtmp, kerv[k][mu][nu][lam] * corr_I[i++]);
      qed_kernel(&qp, ym, xm, kerv);
      i = 0;
      for (int k = 0; k < 6; k++)
        for (int mu = 0; mu < 4; mu++)
          for (int nu = 0; nu < 4; nu++)
            for (int lam = 0; lam < 4; lam++) acc_add(&dtmp, kerv[k][nu][mu][lam] * corr_I[i++]);
      qed_kernel(&qp, xm, xm_mi_ym, kerv);
      i = 0;
      for (int k = 0; k < 6; k++)
        for (int mu = 0; mu < 4; mu++)
          for (int nu = 0; nu < 4; nu++)
            for (int lam = 0; lam < 4; lam++) {
              acc_add(&dtmp, -(kerv[k][lam][nu][mu] * corr_I[i]));
              acc_add(&dtmp, kerv[k][lam][nu][mu] * corr_II[i]);
              i++;
            }
      acc_add(&sum, acc_get(&dtmp));
    }
    part[thread_id()] = sum;
    free(corr_I);
  }
  acc_t total = {0.0, 0.0};
  for (int th = 0; th < nt; ++th) {
    acc_add(&total, part[th].s);
    acc_add(&total, part[th].c);
  }
  free(part);
  return acc_get(&total);
}

/* ---- Contractor::kernel_sum (contract.cpp:104-114), one rank ---------- */
void oracle_kernel_sum(const double* fwd_src, const double* fwd_y, const int gsx[4],
                       const int yv[4], double xunit, double lambda, const int global[4],
                       const int local[4], const int pc[4], double out[2]) {
  double dzu[1728], dzsu[1152], g_dzu[6912], g_dzsu[4608];
  for (int f = 0; f < 2; ++f) {
    memset(dzu, 0, sizeof dzu);
    memset(dzsu, 0, sizeof dzsu);
    oracle_dzu_dzsu(dzu, dzsu, fwd_src, fwd_y, f, pc, gsx, global, local);
    oracle_insert_gammas(dzu, dzsu, g_dzu, g_dzsu);
    out[f] = oracle_4pt(g_dzu, g_dzsu, fwd_src, fwd_y, f, pc, gsx, xunit, yv, lambda,
                        global, local);
  }
}

/* Pass 1 of one flavour, summed into the caller's buffers, then gamma
 * insertion: what compute_dzu_dzsu leaves on the device (contract.cpp:33-81). */
void oracle_g_dzu_dzsu(const double* fwd_src, const double* fwd_y, int iflavor,
                       const int gsx[4], const int global[4], const int local[4],
                       const int pc[4], double* dzu, double* dzsu, double* g_dzu,
                       double* g_dzsu) {
  memset(dzu, 0, sizeof(double) * 1728);
  memset(dzsu, 0, sizeof(double) * 1152);
  oracle_dzu_dzsu(dzu, dzsu, fwd_src, fwd_y, iflavor, pc, gsx, global, local);
  oracle_insert_gammas(dzu, dzsu, g_dzu, g_dzsu);
}

/* ======================================================================
 * 2+2 pieces (kernels/hlbl_kernels/kernels.cu), one rank's part.
 * ==================================================================== */

/* Pi(z)[mu][nu] = Re sum_ia (g_nu g5 w_ia)[ia],
 *   w_ia[ib] = <d_ib, g5 g_mu u_ia>,  u = fwd[iflavor](z), d = fwd[1-iflavor](z)
 * (kernel_pi, kernels.cu:241-294). pi[z*16 + mu*4 + nu]. */
void oracle_pi(const double* fwd, long long V, int iflavor, double* pi) {
#pragma omp parallel for schedule(static)
  for (long long ix = 0; ix < V; ++ix) {
    for (int mu = 0; mu < 4; ++mu)
      for (int nu = 0; nu < 4; ++nu) {
        acc_t tr = {0.0, 0.0};
        for (int ia = 0; ia < 12; ++ia) {
          const double* u = fwd + ((size_t)(iflavor * 12 + ia) * (size_t)V + (size_t)ix) * 24;
          double gu[24], w[24], hw[24];
          apply_gamma(mu, u, gu);
          times_g5(gu);
          for (int ib = 0; ib < 12; ++ib) {
            const double* d = fwd + ((size_t)((1 - iflavor) * 12 + ib) * (size_t)V + (size_t)ix) * 24;
            acc_t re = {0.0, 0.0}, im = {0.0, 0.0};
            for (int c = 0; c < 12; ++c) {
              acc_add(&re, d[2 * c] * gu[2 * c] + d[2 * c + 1] * gu[2 * c + 1]);
              acc_add(&im, d[2 * c] * gu[2 * c + 1] - d[2 * c + 1] * gu[2 * c]);
            }
            w[2 * ib] = acc_get(&re);
            w[2 * ib + 1] = acc_get(&im);
          }
          times_g5(w);
          apply_gamma(nu, w, hw);
          acc_add(&tr, hw[2 * ia]);
        }
        pi[ix * 16 + mu * 4 + nu] = acc_get(&tr);
      }
  }
}

/* P1[rho][sigma][nu][zeta] += sum over this rank's sites z with
 * (z_rho + pc_rho L_rho - gsw_rho) mod G_rho = zeta of Pi(z)[sigma][nu]
 * (kernel_p1, kernels.cu:296-339). p1 is [4][4][4][lmax]. */
void oracle_p1_2p2(const double* pi, const int global[4], const int local[4], const int pc[4],
                   const int gsw[4], int lmax, double* p1) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
  for (int rho = 0; rho < 4; ++rho)
    for (int zr = 0; zr < local[rho]; ++zr) {
      acc_t sum[16];
      memset(sum, 0, sizeof sum);
      for (size_t ix = 0; ix < V; ++ix) {
        int coord[4];
        site_coords(ix, local, coord);
        if (coord[rho] != zr) continue;
        for (int c = 0; c < 16; ++c) acc_add(&sum[c], pi[ix * 16 + c]);
      }
      int const zeta = oracle_mod_pos(zr + local[rho] * pc[rho] - gsw[rho], global[rho]);
      for (int c = 0; c < 16; ++c) p1[(rho * 16 + c) * lmax + zeta] += acc_get(&sum[c]);
    }
}

/* P2_0, P2_1, P3, P4_0, P4_1 of every target (kernels.cu:374-750), this
 * rank's part, added into p234[(t*5 + geom)*64 + rho*16 + sigma*4 + nu]:
 *   y = (target - gsw) mod G, x = (z + pc L - gsw) mod G (per direction),
 *   all kernel arguments mapped to [-L/2, L/2) and scaled by xunit:
 *   P2_0[k][nu] = sum K(x, y)[k][mu][nu][lam]         Pi[mu][lam]
 *   P2_1[k][nu] = sum K(y, x)[k][nu][mu][lam]         Pi[mu][lam]
 *   P3[k][nu]   = sum K(x - y, -y)[k][mu][lam][nu]    Pi[mu][lam]
 *   P4_0[k][nu] = sum K(y - x, -x)[k][nu][lam][mu]    Pi[mu][lam]
 *   P4_1: P4_0's terms times xv[rho] into [rho][sigma], times -xv[sigma]
 *   into [sigma][rho] (xv = the mapped x, unscaled),
 * with k the (rho, sigma) pair, rho < sigma; -y and -x are mapped on their
 * own ((G - y) mod G), as the reference does. */
void oracle_p234(const double* pi, const int global[4], const int local[4], const int pc[4],
                 const int gsw[4], const int* targets, int n_y, double xunit, double lambda,
                 double* p234) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
  int const nt = n_threads();
  hlbl_qed_params qp;
  hlbl_qed_params_init(&qp, lambda);
  acc_t* part = (acc_t*)calloc((size_t)nt * 5 * 64, sizeof(acc_t));
  for (int t = 0; t < n_y; ++t) {
    int y[4];
    double ym[4], ym_minus[4];
    for (int r = 0; r < 4; ++r) {
      y[r] = oracle_mod_pos(targets[4 * t + r] - gsw[r], global[r]);
      ym[r] = oracle_coord_map(y[r], global[r]) * xunit;
      ym_minus[r] = oracle_coord_map((global[r] - y[r]) % global[r], global[r]) * xunit;
    }
    memset(part, 0, sizeof(acc_t) * (size_t)nt * 5 * 64);
#pragma omp parallel
    {
      acc_t* my = part + (size_t)thread_id() * 5 * 64;
      double kerv[6][4][4][4];
#pragma omp for schedule(static)
      for (long long ix = 0; ix < (long long)V; ++ix) {
        int coord[4], xv[4];
        double xm[4], xm_minus[4], xmy[4], ymx[4];
        site_coords((size_t)ix, local, coord);
        for (int r = 0; r < 4; ++r) {
          int const x = oracle_mod_pos(coord[r] + pc[r] * local[r] - gsw[r], global[r]);
          xv[r] = oracle_coord_map(x, global[r]);
          xm[r] = xv[r] * xunit;
          xm_minus[r] = oracle_coord_map((global[r] - x) % global[r], global[r]) * xunit;
          xmy[r] = oracle_coord_map(oracle_mod_pos(x - y[r], global[r]), global[r]) * xunit;
          ymx[r] = oracle_coord_map(oracle_mod_pos(y[r] - x, global[r]), global[r]) * xunit;
        }
        const double* P = pi + ix * 16;
        for (int g = 0; g < 4; ++g) {
          if (g == 0) qed_kernel(&qp, xm, ym, kerv);
          else if (g == 1) qed_kernel(&qp, ym, xm, kerv);
          else if (g == 2) qed_kernel(&qp, xmy, ym_minus, kerv);
          else qed_kernel(&qp, ymx, xm_minus, kerv);
          for (int k = 0; k < 6; ++k) {
            int const rho = comb[k][0], sigma = comb[k][1];
            for (int nu = 0; nu < 4; ++nu) {
              acc_t v = {0.0, 0.0};
              for (int mu = 0; mu < 4; ++mu)
                for (int lam = 0; lam < 4; ++lam) {
                  double const kv = g == 0 ? kerv[k][mu][nu][lam]
                                  : g == 1 ? kerv[k][nu][mu][lam]
                                  : g == 2 ? kerv[k][mu][lam][nu]
                                           : kerv[k][nu][lam][mu];
                  acc_add(&v, kv * P[mu * 4 + lam]);
                }
              double const val = acc_get(&v);
              acc_add(&my[g * 64 + rho * 16 + sigma * 4 + nu], val);
              if (g == 3) {
                acc_add(&my[4 * 64 + rho * 16 + sigma * 4 + nu], xv[rho] * val);
                acc_add(&my[4 * 64 + sigma * 16 + rho * 4 + nu], -(xv[sigma] * val));
              }
            }
          }
        }
      }
    }
    for (int i = 0; i < 5 * 64; ++i) {
      acc_t tot = {0.0, 0.0};
      for (int th = 0; th < nt; ++th) {
        acc_add(&tot, part[(size_t)th * 5 * 64 + i].s);
        acc_add(&tot, part[(size_t)th * 5 * 64 + i].c);
      }
      p234[(size_t)t * 5 * 64 + i] += acc_get(&tot);
    }
  }
  free(part);
}

/* compute_2p2_gpu (kernels.cu:753-870) of one rank, in the per-target
 * layout of Contractor::pieces_2p2 (contract.cpp:116-156):
 * p1 [4][4][4][lmax] and p234 [n_y][5][64], both overwritten with this
 * rank's part (the caller sums over ranks). */
void oracle_pieces_2p2(const double* fwd, int iflavor, const int gsw[4], const int* targets,
                       int n_y, double xunit, double lambda, const int global[4],
                       const int local[4], const int pc[4], double* p1, double* p234) {
  size_t const V = (size_t)local[0] * local[1] * local[2] * local[3];
  int lmax = global[0];
  for (int r = 1; r < 4; ++r) lmax = global[r] > lmax ? global[r] : lmax;
  double* pi = (double*)malloc(sizeof(double) * 16 * (V ? V : 1));
  oracle_pi(fwd, (long long)V, iflavor, pi);
  memset(p1, 0, sizeof(double) * 64 * (size_t)lmax);
  memset(p234, 0, sizeof(double) * 5 * 64 * (size_t)n_y);
  oracle_p1_2p2(pi, global, local, pc, gsw, lmax, p1);
  oracle_p234(pi, global, local, pc, gsw, targets, n_y, xunit, lambda, p234);
  free(pi);
}
