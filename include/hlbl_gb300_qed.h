/*
 * hlbl_gb300_qed.h -- the project's stand-in for the QED kernel L^(Lambda).
 *
 * The reference weights every site of the connected contraction with the KQED
 * library's kernel, QED_Mkernel_L2(0.4, x, y, temps, kerv[6][4][4][4])
 * (kernels/cuda_lattice.cu:266-275, called three times per site at
 * :435, :448, :461). KQED is an external dependency that is not vendored with
 * the reference (https://github.com/RJHudspith/KQED, no commit pinned); its
 * weight functions come from precomputed tables that are not available to this
 * project. This header defines a STAND-IN with the same signature, the same
 * index structure and the same shape of computation:
 *
 *   - six scalar weight functions w_j(|x|, xhat.yhat, |y|) (KQED also reduces
 *     the kernel to a handful of scalar functions of these three invariants);
 *   - an exact tensor assembly of kerv[k][mu][nu][lambda] from w_j, x and y,
 *     antisymmetric in the (rho, sigma) pair k of the reference's idx_comb
 *     order (cuda_lattice.cu:52-60): (0,1) (0,2) (0,3) (1,2) (1,3) (2,3).
 *
 * The weight functions are 16-node Gauss-Legendre quadratures over a Feynman
 * parameter u in [0,1]:
 *
 *   w_j(X, c, Y) = sum_i g_i h_j(u_i) exp(-m_j sqrt(R_i^2 + Lambda^2)) / (1 + R_i^2)
 *   R_i^2        = u_i^2 X^2 + (1-u_i)^2 Y^2 - 2 u_i (1-u_i) X Y c   (>= 0)
 *   h_j(u)       = 1, u, 1-u, u(1-u), u^2, (1-u)^2
 *   m_j          = 0.6 + 0.2 j            (units of the muon mass)
 *
 * with X = |x|, Y = |y|, c = x.y/(|x||y|) (0 when x or y is 0). The quadrature
 * IS the definition (it is not an approximation of anything), so the exact
 * FP64 weight is reproducible to rounding on every platform. Its cost (96
 * exponentials per evaluation) stands in for KQED's table interpolation.
 * Results computed with it are NOT physics: they pin the contraction algebra,
 * the coordinate rules and the reductions, not the value of a_mu.
 *
 * Tensor assembly (d = x - y, s = x + y, [rho sigma] antisymmetrised):
 *   kerv = w0 (d_{mu rho} d_{nu sigma} - d_{mu sigma} d_{nu rho}) x_lambda
 *        + w1 (d_{mu rho} d_{lambda sigma} - d_{mu sigma} d_{lambda rho}) y_nu
 *        + w2 (d_{nu rho} d_{lambda sigma} - d_{nu sigma} d_{lambda rho}) d_mu
 *        + w3 (x_rho y_sigma - x_sigma y_rho) delta_{mu nu} s_lambda
 *        + w4 (x_rho delta_{sigma mu} - x_sigma delta_{rho mu}) y_nu y_lambda
 *        + w5 (y_rho delta_{sigma lambda} - y_sigma delta_{rho lambda}) x_mu x_nu
 * (d_{ab} above is the Kronecker delta.)
 *
 * Compiles as C (gcc), C++ (g++) and CUDA (nvcc, host and device).
 */
#ifndef HLBL_GB300_QED_H
#define HLBL_GB300_QED_H

#include <math.h>

#if defined(__CUDACC__)
#define HLBL_QED_HD __host__ __device__ __forceinline__
#else
#define HLBL_QED_HD static inline
#endif

#define HLBL_QED_NW 6  /* scalar weight functions */
#define HLBL_QED_NQ 16 /* quadrature nodes */

#ifdef __cplusplus
extern "C" {
#endif

/* Everything the weight needs; plays the role of KQED's QED_kernel_temps. */
typedef struct hlbl_qed_params {
  double lambda;                /* Lambda of L^(Lambda); the reference passes 0.4 */
  double mass[HLBL_QED_NW];     /* m_j */
  double node[HLBL_QED_NQ];     /* u_i, Gauss-Legendre nodes on [0,1] */
  double weight[HLBL_QED_NQ];   /* g_i, their weights (sum to 1) */
} hlbl_qed_params;

/* The (rho, sigma) pair of k, in the reference's idx_comb order. */
HLBL_QED_HD int hlbl_qed_rho(int k) { return k < 3 ? 0 : (k < 5 ? 1 : 2); }
HLBL_QED_HD int hlbl_qed_sigma(int k) { return k < 3 ? k + 1 : (k < 5 ? k - 1 : 3); }

/* Host: the parameters for a given Lambda. Nodes by Newton iteration on the
 * Legendre polynomial P_16 (three-term recurrence), mapped to [0,1]. */
static inline void hlbl_qed_params_init(hlbl_qed_params* p, double lambda) {
  const int n = HLBL_QED_NQ;
  const double pi = 3.14159265358979323846;
  p->lambda = lambda;
  for (int j = 0; j < HLBL_QED_NW; ++j) p->mass[j] = 0.6 + 0.2 * j;
  for (int i = 0; i < n; ++i) {
    double t = cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = t;
      for (int l = 2; l <= n; ++l) {
        double p2 = ((2.0 * l - 1.0) * t * p1 - (l - 1.0) * p0) / l;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (t * p1 - p0) / (t * t - 1.0);
      double dt = p1 / dp;
      t -= dt;
      if (fabs(dt) < 1e-16) break;
    }
    {
      double p0 = 1.0, p1 = t;
      for (int l = 2; l <= n; ++l) {
        double p2 = ((2.0 * l - 1.0) * t * p1 - (l - 1.0) * p0) / l;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (t * p1 - p0) / (t * t - 1.0);
    }
    /* weight on [-1,1] is 2/((1-t^2) P'^2); on [0,1] half of it */
    p->node[i] = 0.5 * (1.0 - t);
    p->weight[i] = 1.0 / ((1.0 - t * t) * dp * dp);
  }
}

/* The three invariants of the pair (x, y): |x|, cos(x, y), |y|. */
HLBL_QED_HD void hlbl_qed_invariants(const double x[4], const double y[4],
                                     double* X, double* c, double* Y) {
  double xx = 0, yy = 0, xy = 0;
  for (int a = 0; a < 4; ++a) {
    xx += x[a] * x[a];
    yy += y[a] * y[a];
    xy += x[a] * y[a];
  }
  *X = sqrt(xx);
  *Y = sqrt(yy);
  double const den = (*X) * (*Y);
  double cc = den > 0 ? xy / den : 0.0;
  cc = cc > 1.0 ? 1.0 : (cc < -1.0 ? -1.0 : cc);
  *c = cc;
}

/* The six weight functions at (X, c, Y). */
HLBL_QED_HD void hlbl_qed_weights(const hlbl_qed_params* p, double X, double c,
                                  double Y, double w[HLBL_QED_NW]) {
  for (int j = 0; j < HLBL_QED_NW; ++j) w[j] = 0.0;
  double const l2 = p->lambda * p->lambda;
  for (int i = 0; i < HLBL_QED_NQ; ++i) {
    double const u = p->node[i], v = 1.0 - u;
    double r2 = u * u * X * X + v * v * Y * Y - 2.0 * u * v * X * Y * c;
    r2 = r2 > 0 ? r2 : 0.0;
    double const g = p->weight[i] / (1.0 + r2);
    double const r = sqrt(r2 + l2);
    double const h[HLBL_QED_NW] = {1.0, u, v, u * v, u * u, v * v};
    for (int j = 0; j < HLBL_QED_NW; ++j) w[j] += g * h[j] * exp(-p->mass[j] * r);
  }
}

/* One component kerv[k][mu][nu][lam] of the tensor assembly, given w. */
HLBL_QED_HD double hlbl_qed_entry(const double w[HLBL_QED_NW], const double x[4],
                                  const double y[4], int k, int mu, int nu, int lam) {
  int const r = hlbl_qed_rho(k), s = hlbl_qed_sigma(k);
  double const dmr = mu == r, dms = mu == s, dnr = nu == r, dns = nu == s;
  double const dlr = lam == r, dls = lam == s, dmn = mu == nu;
  double v = w[0] * (dmr * dns - dms * dnr) * x[lam];
  v += w[1] * (dmr * dls - dms * dlr) * y[nu];
  v += w[2] * (dnr * dls - dns * dlr) * (x[mu] - y[mu]);
  v += w[3] * (x[r] * y[s] - x[s] * y[r]) * dmn * (x[lam] + y[lam]);
  v += w[4] * (x[r] * dms - x[s] * dmr) * y[nu] * y[lam];
  v += w[5] * (y[r] * dls - y[s] * dlr) * x[mu] * x[nu];
  return v;
}

/* The whole tensor, KQED's output layout kerv[6][4][4][4]. */
HLBL_QED_HD void hlbl_qed_kernel(const hlbl_qed_params* p, const double x[4],
                                 const double y[4], double kerv[6][4][4][4]) {
  double X, c, Y, w[HLBL_QED_NW];
  hlbl_qed_invariants(x, y, &X, &c, &Y);
  hlbl_qed_weights(p, X, c, Y, w);
  for (int k = 0; k < 6; ++k)
    for (int mu = 0; mu < 4; ++mu)
      for (int nu = 0; nu < 4; ++nu)
        for (int lam = 0; lam < 4; ++lam)
          kerv[k][mu][nu][lam] = hlbl_qed_entry(w, x, y, k, mu, nu, lam);
}

/* ---- a second test weight with no closed form ------------------------------
 *
 * The stand-in above is a sum of Kronecker structures, and the library's
 * fast contraction paths exploit that. To check the paths that accept ANY
 * tensor kerv[6][4][4][4] (a provider with QED_Mkernel_L2's signature), this
 * dense test weight gives every one of the 384 entries its own seeded
 * combination of thirteen smooth functions of the two arguments:
 *
 *   kerv[i](x, y) = sum_b A[b][i] phi_b(x, y),   i = ((k*4 + mu)*4 + nu)*4 + lam
 *   phi_0 = g, phi_{1+a} = g x_a, phi_{5+a} = g y_a, phi_{9+a} = g x_a y_a
 *   g     = 1 / (1 + |x|^2 + |y|^2 + |x - y|^2 / 2)
 *
 * with A[b][i] uniform in [-1, 1) from a splitmix64 hash of (seed, b, i)
 * (exact in binary, the same on every platform). The entries share no
 * index structure, so no contraction of the tensor has a shortcut. Like the
 * stand-in it is test physics only. */
#define HLBL_QED_NK 384       /* entries of kerv[6][4][4][4] */
#define HLBL_QED_DENSE_NB 13  /* basis functions */

/* A[b][i], row-major: HLBL_QED_DENSE_NB x HLBL_QED_NK doubles. */
static inline void hlbl_qed_dense_init(double* table, unsigned long long seed) {
  for (int i = 0; i < HLBL_QED_DENSE_NB * HLBL_QED_NK; ++i) {
    unsigned long long x = seed * 0x9E3779B97F4A7C15ULL + (unsigned long long)i;
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    x ^= x >> 31;
    table[i] = (double)(x >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  }
}

/* The thirteen basis functions at (x, y). */
HLBL_QED_HD void hlbl_qed_dense_basis(const double x[4], const double y[4],
                                      double phi[HLBL_QED_DENSE_NB]) {
  double xx = 0, yy = 0, dd = 0;
  for (int a = 0; a < 4; ++a) {
    double const d = x[a] - y[a];
    xx += x[a] * x[a];
    yy += y[a] * y[a];
    dd += d * d;
  }
  double const g = 1.0 / (1.0 + xx + yy + 0.5 * dd);
  phi[0] = g;
  for (int a = 0; a < 4; ++a) {
    phi[1 + a] = g * x[a];
    phi[5 + a] = g * y[a];
    phi[9 + a] = g * x[a] * y[a];
  }
}

/* Entry i of the tensor from the basis values. */
HLBL_QED_HD double hlbl_qed_dense_entry(const double* table,
                                        const double phi[HLBL_QED_DENSE_NB], int i) {
  double v = 0.0;
  for (int b = 0; b < HLBL_QED_DENSE_NB; ++b) v += table[b * HLBL_QED_NK + i] * phi[b];
  return v;
}

/* The whole tensor, KQED's output layout kerv[6][4][4][4]. */
HLBL_QED_HD void hlbl_qed_dense_kernel(const double* table, const double x[4],
                                       const double y[4], double kerv[6][4][4][4]) {
  double phi[HLBL_QED_DENSE_NB];
  hlbl_qed_dense_basis(x, y, phi);
  double* k = &kerv[0][0][0][0];
  for (int i = 0; i < HLBL_QED_NK; ++i) k[i] = hlbl_qed_dense_entry(table, phi, i);
}

#ifdef __cplusplus
}
#endif

#endif /* HLBL_GB300_QED_H */
