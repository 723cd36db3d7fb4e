// pieces_2p2.cu -- the 2+2 pieces of one source w (compute_2p2_gpu,
// kernels/hlbl_kernels/kernels.cu:753-870; Contractor::pieces_2p2,
// src/contract.cpp:116-156) on one GPU:
//
//   pi_kernel       Pi(z)[mu][nu] for every local site          (kernel_pi :241-294)
//   p1_2p2_kernel   P1[rho][sigma][nu][zeta] slab sums of Pi     (kernel_p1 :296-339)
//   p234_kernel<G>  per target, partial sums per CTA of          (kernel_p20 :374-458,
//                   G = 0: P2_0, 1: P2_1, 2: P3, 3: P4_0 + P4_1   kernel_p21 :461-545,
//                                                                kernel_p3 :548-643,
//                                                                kernel_p4 :646-750)
//   p234_reduce     the CTA partials summed in FP64, in either output layout
//
// Precision HLBL_FP64 computes everything in FP64 (the reference's
// arithmetic). HLBL_FP32 forms Pi's products in FP32 from the FP64 block,
// evaluates the stand-in QED weight by the FP32 quadrature (FP64 where an
// argument is shorter than r64, near the origin), contracts in FP32 and
// sums per thread in FP32, per CTA and across CTAs in FP64.
//
// Pi. With the cvc gamma matrices as monomial spin matrices
// ((g_m v)[s] = i^ph(m,s) v[src(m,s)]), kernel_pi's
//   Pi[mu][nu] = Re sum_ia (g_nu g5 w_ia)[ia],  w_ia[ib] = <d_ib, g5 g_mu u_ia>
// (u = fwd[iflavor], d = fwd[1-iflavor], rows ia = (s, a): spin s, colour a)
// becomes a sum over the sixteen spin pairs (s, s2) of
//   Re(i^p Z),  Z = sum_{a,c} conj(d[(src(nu,s), a)][(s2, c)]) u[(s, a)][(src(mu,s2), c)],
//   p = ph(g_nu g5, s) + ph(g5 g_mu, s2).
// src(nu, s) takes two values over nu (s^2, 3-s), so a site needs 64 traces
// Z: 16 threads per site form four each (one (s, s2), 144 FMAs), then each
// of the 16 threads sums its (mu, nu)'s sixteen; the site's 24 rows and its
// traces are staged in shared memory.
//
// P2/P3/P4. The stand-in kernel (include/hlbl_gb300_qed.h) is
//   K[k][m][n][l] = sum_j w_j T_j(a, b)[k][m][n][l]
// with T_j products of Kronecker deltas and the argument vectors a, b. Each
// geometry contracts two of K's three Lorentz indices with Pi (or Pi^T) and
// keeps the third: contracting the T_j in closed form leaves four mat-vecs
// of Pi with a and b and a few scalars (contract<F> below), instead of the
// 384-entry tensor and 384 products per evaluation.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "hlbl_device.cuh"
#include "hlbl_gb300.h"
#include "hlbl_internal.h"
#include "pieces_2p2.h"
#include "qed_f32.cuh"
#include "qed_provider.cuh"

namespace hg {
namespace p22 {

// ---- Pi --------------------------------------------------------------------
constexpr int kPiSites = 8;                 // sites per tile
constexpr int kPiThreads = 16 * kPiSites;   // one thread per (site, mu, nu)

// Site records rec[V][kRec]: Pi[mu*4 + nu] at 0..15, then the site's mapped
// position relative to the source, coord_map((z + pc L - gsw) mod G), at
// 16..19 (small integers, exact in T).
constexpr int kRec = 20;

// Input: the FP64 block fwd, or (T = float, x32 not null) its FP32 tile copy.
// a site's 24 staged rows, padded by 16 bytes so that the 8 sites of a tile
// start in different banks
constexpr int kPiRow = 12 * 24 + 4;
// staging loads per thread and tile from the FP32 tile copy: 24 rows x 6
// groups x 8 sites of float4
constexpr int kPiLd32 = 24 * 6 * kPiSites / kPiThreads;
static_assert(kPiLd32 * kPiThreads == 24 * 6 * kPiSites, "");

// Input: the FP64 block fwd, or (FROM32) its FP32 tile copy x32.
template <typename T, bool FROM32>
__global__ void __launch_bounds__(kPiThreads, FROM32 ? 4 : 1) pi_kernel(const double* __restrict__ fwd,
                                                        const float* __restrict__ x32, Geometry geo,
                                                        int4 gsw, int iflavor, T* __restrict__ rec) {
  static_assert(!FROM32 || sizeof(T) == 4, "the FP32 tile copy feeds the FP32 path");
  long long const V = geo.V;
  __shared__ __align__(16) T su[kPiSites][kPiRow];
  __shared__ __align__(16) T sd[kPiSites][kPiRow];
  __shared__ __align__(16) T sz[kPiSites][64][2];
  int const t = threadIdx.x, st = t >> 4, mu = (t >> 2) & 3, nu = t & 3;
  long long const ntiles = (V + kPiSites - 1) / kPiSites;
  long long const nt32 = (V + 31) / 32;
  // the FP32 tile copy: the staging loads of tile `tile` into registers
  float4 r32[FROM32 ? kPiLd32 : 1];
  auto load = [&](long long tile) {
    long long const s0 = tile * kPiSites;
    if constexpr (FROM32) {
      // a row's 8 sites (inside one 16-site half) are six runs of 8 x 16 bytes
#pragma unroll
      for (int q = 0; q < kPiLd32; ++q) {
        int const i = t + q * kPiThreads;
        int const row = i / (6 * kPiSites), k = i % (6 * kPiSites), c4 = k / kPiSites, sl = k % kPiSites;
        int const ia = row % 12, f = row < 12 ? iflavor : 1 - iflavor;
        long long const s = s0 + sl;  // < the padded length of the copy
        r32[q] = __ldg(reinterpret_cast<const float4*>(
            x32 + ((size_t)(f * 12 + ia) * nt32 + (size_t)(s >> 5)) * 768 + f32_tile_off((int)(s & 31), c4)));
      }
    }
  };
  // the FP32 tile copy: the next tile's loads are in flight while this one
  // is computed; the FP64 block (twice the registers): loaded when needed
  if (FROM32 && blockIdx.x < ntiles) load(blockIdx.x);
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    long long const s0 = tile * kPiSites;
    int const ns = (int)min((long long)kPiSites, V - s0);

    // registers -> shared (u rows: flavour iflavor, d rows: 1 - iflavor)
    if constexpr (FROM32) {
#pragma unroll
      for (int q = 0; q < kPiLd32; ++q) {
        int const i = t + q * kPiThreads;
        int const row = i / (6 * kPiSites), k = i % (6 * kPiSites), c4 = k / kPiSites, sl = k % kPiSites;
        T* dst = (row < 12 ? su[sl] : sd[sl]) + (row % 12) * 24 + 4 * c4;
        *reinterpret_cast<float4*>(dst) = r32[q];
      }
    } else {
      // the FP64 block: 24 rows x the tile's sites as double2, straight to shared
#pragma unroll 6
      for (int i = t; i < 24 * kPiSites * 12; i += kPiThreads) {
        int const row = i / (kPiSites * 12), j = i % (kPiSites * 12), s = j / 12, c2 = j % 12;
        int const ia = row % 12, f = row < 12 ? iflavor : 1 - iflavor;
        double2 v = make_double2(0.0, 0.0);
        if (s < ns) v = __ldg(reinterpret_cast<const double2*>(fwd + ((size_t)(f * 12 + ia) * V + s0 + s) * 24) + c2);
        T* dst = (row < 12 ? su[s] : sd[s]) + ia * 24 + 2 * c2;
        if constexpr (sizeof(T) == 4) {
          // on the integer pipe, not the FP64 pipe
          *reinterpret_cast<float2*>(dst) = make_float2(f64_to_f32(v.x), f64_to_f32(v.y));
        } else {
          *reinterpret_cast<double2*>(dst) = v;
        }
      }
    }
    __syncthreads();
    if (FROM32 && tile + gridDim.x < ntiles) load(tile + gridDim.x);
    // phase 1, thread (site, s, s2): the four traces
    //   Z[jb][jd] = sum_{a,c} conj(d[(sb, a)][(s2, c)]) u[(s, a)][(sd, c)],
    //   sb = s^2 (jb = 0) or 3-s (jb = 1), sd = s2^2 (jd = 0) or 3-s2 (jd = 1)
    if (st < ns) {
      int const s = (t >> 2) & 3, s2 = t & 3;
      const T* U = su[st];
      const T* D = sd[st];
      T zr[2][2], zi[2][2];
#pragma unroll
      for (int jb = 0; jb < 2; ++jb) {
        int const sb = jb ? 3 - s : (s ^ 2);
#pragma unroll
        for (int jd = 0; jd < 2; ++jd) {
          int const sdd = jd ? 3 - s2 : (s2 ^ 2);
          T re = T(0), im = T(0);
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const T* dp = D + (3 * sb + a) * 24 + 2 * (3 * s2 + c);
              const T* up = U + (3 * s + a) * 24 + 2 * (3 * sdd + c);
              T const dr = dp[0], di = dp[1], ur = up[0], ui = up[1];
              re += dr * ur + di * ui;
              im += dr * ui - di * ur;
            }
          zr[jb][jd] = re;
          zi[jb][jd] = im;
        }
      }
#pragma unroll
      for (int jb = 0; jb < 2; ++jb)
#pragma unroll
        for (int jd = 0; jd < 2; ++jd) {
          sz[st][(s * 4 + s2) * 4 + jb * 2 + jd][0] = zr[jb][jd];
          sz[st][(s * 4 + s2) * 4 + jb * 2 + jd][1] = zi[jb][jd];
        }
    }
    __syncthreads();
    // phase 2, thread (site, mu, nu): Pi = sum_{s,s2} Re(i^p Z[s][s2][jb(nu)][jd(mu)]),
    // p = ph(g_nu g5, s) + ph(g5 g_mu, s2); g_0, g_3 map spin s to s^2, g_1, g_2 to 3-s
    if (st < ns) {
      int const jb = (nu == 0 || nu == 3) ? 0 : 1, jd = (mu == 0 || mu == 3) ? 0 : 1;
      T acc = T(0);
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        int const pn = gg5_ph(nu, s);
#pragma unroll
        for (int s2 = 0; s2 < 4; ++s2) {
          int const p = (pn + g5g_ph(mu, s2)) & 3;
          const T* z = sz[st][(s * 4 + s2) * 4 + jb * 2 + jd];
          // Re(i^p Z): +Re Z, -Im Z, -Re Z, +Im Z
          T const v = (p & 1) ? z[1] : z[0];
          acc += (p == 1 || p == 2) ? -v : v;
        }
      }
      rec[(s0 + st) * kRec + mu * 4 + nu] = acc;
    }
    if (t < ns) {
      int const gw[4] = {gsw.x, gsw.y, gsw.z, gsw.w};
      int x[4];
      rel_coords(geo, gw, s0 + t, x);
#pragma unroll
      for (int r = 0; r < 4; ++r) rec[(s0 + t) * kRec + 16 + r] = (T)coord_map(x[r], geo.global[r]);
    }
    __syncthreads();
  }
}

// ---- P1 --------------------------------------------------------------------
constexpr int kP1Threads = 256;
constexpr int kP1Split = 64;  // CTAs per slab

// blockIdx.x = (rho, zr), zr a local coordinate along rho; blockIdx.y = the
// slab's part: the CTA sums Pi over every kP1Split-th group of the slab's
// sites, part[(blockIdx.x * kP1Split + blockIdx.y) * 16 + sigma*4 + nu].
template <typename T>
__global__ void __launch_bounds__(kP1Threads) p1_2p2_kernel(const T* __restrict__ rec, Geometry geo,
                                                            double* __restrict__ part) {
  int b = blockIdx.x, rho = 0;
  while (rho < 3 && b >= geo.local[rho]) {
    b -= geo.local[rho];
    ++rho;
  }
  int const zr = b;
  int const d0 = rho == 0 ? 1 : 0, d1 = rho <= 1 ? 2 : 1, d2 = rho <= 2 ? 3 : 2;
  // the slab's sites number V / L_rho < 2^31 (a single GPU's lattice)
  unsigned const L1 = geo.local[d1], L2 = geo.local[d2], L12 = L1 * L2;
  unsigned const nslab = (unsigned)(geo.V / geo.local[rho]);
  int const c = threadIdx.x & 15, grp = threadIdx.x >> 4;
  constexpr int kGroups = kP1Threads / 16;
  // FP32 records: compensated FP32 sums, converted once (FP64 adds would
  // run on the FP64 pipe); FP64 records: FP64 sums
  std::conditional_t<sizeof(T) == 4, KahanF, double> sum{};
  for (unsigned i = blockIdx.y * kGroups + grp; i < nslab; i += kP1Split * kGroups) {
    int z[4];
    z[rho] = zr;
    z[d0] = (int)(i / L12);
    z[d1] = (int)((i / L2) % L1);
    z[d2] = (int)(i % L2);
    long long const site =
        (((long long)z[0] * geo.local[1] + z[1]) * geo.local[2] + z[2]) * geo.local[3] + z[3];
    if constexpr (sizeof(T) == 4) sum.add(rec[site * kRec + c]);
    else sum += rec[site * kRec + c];
  }
  double acc;
  if constexpr (sizeof(T) == 4) acc = sum.get();
  else acc = sum;
  __shared__ double red[kGroups][17];
  red[grp][c] = acc;
  __syncthreads();
  if (threadIdx.x < 16) {
    double s = 0.0;
    for (int g = 0; g < kGroups; ++g) s += red[g][threadIdx.x];
    part[((size_t)blockIdx.x * kP1Split + blockIdx.y) * 16 + threadIdx.x] = s;
  }
}

// P1[rho][sigma][nu][zeta] of slab blockIdx.x: the sum of its parts, at
// zeta = (zr + pc L - gsw) mod G (kernel_p1, kernels.cu:330-338)
__global__ void p1_2p2_finish_kernel(const double* __restrict__ part, Geometry geo, int4 gsw, int lmax,
                                     double* __restrict__ p1) {
  int b = blockIdx.x, rho = 0;
  while (rho < 3 && b >= geo.local[rho]) {
    b -= geo.local[rho];
    ++rho;
  }
  int const c = threadIdx.x;
  double s = 0.0;
  for (int q = 0; q < kP1Split; ++q) s += part[((size_t)blockIdx.x * kP1Split + q) * 16 + c];
  int const gw[4] = {gsw.x, gsw.y, gsw.z, gsw.w};
  int const zeta = mod_pos(b + geo.local[rho] * geo.pc[rho] - gw[rho], geo.global[rho]);
  p1[(size_t)(rho * 16 + c) * lmax + zeta] = s;
}

// ---- P2_0, P2_1, P3, P4 ----------------------------------------------------
constexpr int kP234Threads = 128;

// The closed-form contraction of the stand-in kernel K(a, b) with a 4x4
// matrix M over two of its Lorentz indices, the third (f) kept, for the six
// pairs k = (r, s):
//   F = 1: v[k][f] = sum_{n,l} K[k][f][n][l] M[n][l]
//   F = 2: v[k][f] = sum_{m,l} K[k][m][f][l] M[m][l]
//   F = 3: v[k][f] = sum_{m,n} K[k][m][n][f] M[m][n]
// TR: M = P^T instead of P. v[k*4 + f].
template <typename T, int F, bool TR>
__device__ __forceinline__ void contract(const T* a, const T* b, const T* w, const T* P, T* v) {
  auto M = [&](int i, int j) -> T { return TR ? P[j * 4 + i] : P[i * 4 + j]; };
  T Ma[4], Mb[4], aM[4], bM[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    Ma[i] = M(i, 0) * a[0] + M(i, 1) * a[1] + M(i, 2) * a[2] + M(i, 3) * a[3];
    Mb[i] = M(i, 0) * b[0] + M(i, 1) * b[1] + M(i, 2) * b[2] + M(i, 3) * b[3];
    aM[i] = a[0] * M(0, i) + a[1] * M(1, i) + a[2] * M(2, i) + a[3] * M(3, i);
    bM[i] = b[0] * M(0, i) + b[1] * M(1, i) + b[2] * M(2, i) + b[3] * M(3, i);
  }
  T const tr = M(0, 0) + M(1, 1) + M(2, 2) + M(3, 3);
  T const bMb = b[0] * Mb[0] + b[1] * Mb[1] + b[2] * Mb[2] + b[3] * Mb[3];
  T const aMa = a[0] * Ma[0] + a[1] * Ma[1] + a[2] * Ma[2] + a[3] * Ma[3];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    int const r = comb_rho(k), s = comb_sigma(k);
    T const A = a[r] * b[s] - a[s] * b[r];
    T const asym = M(r, s) - M(s, r);
    T const c5 = b[r] * aM[s] - b[s] * aM[r];
    T const c4 = a[r] * Mb[s] - a[s] * Mb[r];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      T const fr = f == r ? T(1) : T(0), fs = f == s ? T(1) : T(0);
      T val;
      if constexpr (F == 1) {
        val = w[0] * (fr * Ma[s] - fs * Ma[r]) + w[1] * (fr * bM[s] - fs * bM[r]) +
              w[2] * (a[f] - b[f]) * asym + w[3] * A * (Ma[f] + Mb[f]) +
              w[4] * (fs * a[r] - fr * a[s]) * bMb + w[5] * a[f] * c5;
      } else if constexpr (F == 2) {
        val = w[0] * (fs * Ma[r] - fr * Ma[s]) + w[1] * b[f] * asym +
              w[2] * (fr * (aM[s] - bM[s]) - fs * (aM[r] - bM[r])) + w[3] * A * (Ma[f] + Mb[f]) +
              w[4] * b[f] * c4 + w[5] * a[f] * c5;
      } else {
        val = w[0] * a[f] * asym + w[1] * (fs * Mb[r] - fr * Mb[s]) +
              w[2] * (fs * (aM[r] - bM[r]) - fr * (aM[s] - bM[s])) + w[3] * A * (a[f] + b[f]) * tr +
              w[4] * b[f] * c4 + w[5] * (fs * b[r] - fr * b[s]) * aMa;
      }
      v[k * 4 + f] = val;
    }
  }
}

template <typename T>
__device__ __forceinline__ void weights(const P234Args& p, const T* a, const T* b, T w[6]) {
  if constexpr (sizeof(T) == 8) {
    double X, c, Y;
    hlbl_qed_invariants(a, b, &X, &c, &Y);
    hlbl_qed_weights(&p.qp, X, c, Y, w);
  } else {
    float xx = 0.f, yy = 0.f, xy = 0.f;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      xx = fmaf(a[r], a[r], xx);
      yy = fmaf(b[r], b[r], yy);
      xy = fmaf(a[r], b[r], xy);
    }
    float const X = sqrtf(xx), Y = sqrtf(yy);
    if (fminf(X, Y) < p.r64f) {
      // near the origin: the FP64 weight from the FP64 arguments
      double ad[4], bd[4], Xd, cd, Yd, wd[6];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        ad[r] = (double)a[r];
        bd[r] = (double)b[r];
      }
      hlbl_qed_invariants(ad, bd, &Xd, &cd, &Yd);
      hlbl_qed_weights(&p.qp, Xd, cd, Yd, wd);
#pragma unroll
      for (int j = 0; j < 6; ++j) w[j] = (float)wd[j];
    } else {
      float const den = X * Y;
      float c = den > 0.f ? xy / den : 0.f;
      c = fminf(1.f, fmaxf(-1.f, c));
      if (p.qf.geometric) weights_f32<true>(p.qf, X, c, Y, w);
      else weights_f32<false>(p.qf, X, c, Y, w);
    }
  }
}

// (r, s) with r < s -> k
__host__ __device__ constexpr int comb_index(int r, int s) { return r == 0 ? s - 1 : (r == 1 ? s + 1 : 5); }

// The stand-in's closed-form contraction (the fast variant; contract above).
struct ClosedStandIn {};

// Geometry G's contraction of ANY QED kernel (a provider, qed_provider.cuh)
// with Pi, entry by entry (kernel_p20/p21/p3/p4's index order,
// kernels.cu:374-750), the kept index f:
//   G = 0: v[k][f] = sum_{m,l} K[k][m][f][l] P[m][l]   (P2_0)
//   G = 1: v[k][f] = sum_{n,l} K[k][f][n][l] P[n][l]   (P2_1)
//   G = 2: v[k][f] = sum_{m,n} K[k][m][n][f] P[m][n]   (P3)
//   G = 3: v[k][f] = sum_{n,l} K[k][f][n][l] P[l][n]   (P4)
// 384 entries per evaluation.
template <typename T, int G, class Q>
__device__ __forceinline__ void generic_contract(const Q& prov, const T* a, const T* b, const T* P, T* v) {
  double ad[4], bd[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    ad[r] = (double)a[r];
    bd[r] = (double)b[r];
  }
  T st[Q::kState];
  prov.template prepare<T>(ad, bd, st);
  for (int k = 0; k < 6; ++k) {
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      T acc = T(0);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          int const idx = G == 0 ? kerv_index(k, i, f, j)
                        : G == 2 ? kerv_index(k, i, j, f)
                                 : kerv_index(k, f, i, j);
          T const m = G == 3 ? P[j * 4 + i] : P[i * 4 + j];
          acc = fma(prov.template entry<T>(st, idx), m, acc);
        }
      v[k * 4 + f] = acc;
    }
  }
}

// Geometry G of every target of the launch, partial sums of this CTA:
// part[((t * 5 + slot) * pstride + blockIdx.x) * 64 + rho*16 + sigma*4 + nu].
// Q: ClosedStandIn (the stand-in's closed form, the weights from p.qp) or a
// provider (any QED kernel, generic_contract).
template <class Q>
constexpr int p234_state() {
  if constexpr (std::is_same_v<Q, ClosedStandIn>) return 0;
  else return Q::kState;
}
// FP32: four CTAs per SM (three for G = 3 and its 72 sums); FP64 and
// whole-tensor providers (a linked KQED's device function brings its own
// register count, which a tighter bound would conflict with): one
template <typename T, int G, class Q>
constexpr int p234_min_ctas() {
  return (sizeof(T) == 4 && p234_state<Q>() <= 64) ? (G == 3 ? 3 : 4) : 1;
}

template <typename T, int G, class Q>
__global__ void __launch_bounds__(kP234Threads, p234_min_ctas<T, G, Q>())
    p234_kernel(P234Args p, Q prov, const T* __restrict__ rec, int pstride, double* __restrict__ part) {
  constexpr int NA = G == 3 ? 72 : 24;
  constexpr int NW = kP234Threads / 32;
  __shared__ double red[NW][NA];
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long const stride = (long long)gridDim.x * blockDim.x;
  T const xu = (T)p.xunit;
  // per direction: L, floor(L/2) and -(L - floor(L/2)): a difference d of
  // two mapped coordinates, |d| < L, maps to [-(L - h), h) as
  // coord_map(mod_pos(d, L), L) does, in floating point (exact integers)
  T Lf[4], hf[4], lof[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int const L = p.geo.global[r];
    Lf[r] = (T)L;
    hf[r] = (T)(L / 2);
    lof[r] = (T)(L / 2 - L);
  }
  auto wrap = [&](T d, int r) -> T { return d >= hf[r] ? d - Lf[r] : (d < lof[r] ? d + Lf[r] : d); };
  for (int t = 0; t < p.n_t; ++t) {
    T yv[4], ym[4], ym_minus[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      yv[r] = (T)coord_map(p.y[t][r], p.geo.global[r]);
      ym[r] = yv[r] * xu;
      ym_minus[r] = wrap(-yv[r], r) * xu;
    }
    T acc[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) acc[i] = T(0);
    for (long long site = blockIdx.x * (long long)blockDim.x + threadIdx.x; site < p.geo.V; site += stride) {
      T P[16], xv[4];
      if constexpr (sizeof(T) == 4) {
        const float4* q = reinterpret_cast<const float4*>(rec + site * kRec);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float4 const v = __ldg(q + i);
          P[4 * i] = v.x; P[4 * i + 1] = v.y; P[4 * i + 2] = v.z; P[4 * i + 3] = v.w;
        }
        float4 const v = __ldg(q + 4);
        xv[0] = v.x; xv[1] = v.y; xv[2] = v.z; xv[3] = v.w;
      } else {
        const double2* q = reinterpret_cast<const double2*>(rec + site * kRec);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          double2 const v = __ldg(q + i);
          P[2 * i] = v.x; P[2 * i + 1] = v.y;
        }
        double2 const u = __ldg(q + 8), v = __ldg(q + 9);
        xv[0] = u.x; xv[1] = u.y; xv[2] = v.x; xv[3] = v.y;
      }
      T a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if constexpr (G == 0) {
          a[r] = xv[r] * xu;
          b[r] = ym[r];
        } else if constexpr (G == 1) {
          a[r] = ym[r];
          b[r] = xv[r] * xu;
        } else if constexpr (G == 2) {
          a[r] = wrap(xv[r] - yv[r], r) * xu;
          b[r] = ym_minus[r];
        } else {
          a[r] = wrap(yv[r] - xv[r], r) * xu;
          b[r] = wrap(-xv[r], r) * xu;
        }
      }
      T v[24];
      if constexpr (std::is_same_v<Q, ClosedStandIn>) {
        T w[6];
        weights<T>(p, a, b, w);
        if constexpr (G == 0) contract<T, 2, false>(a, b, w, P, v);
        else if constexpr (G == 1) contract<T, 1, false>(a, b, w, P, v);
        else if constexpr (G == 2) contract<T, 3, false>(a, b, w, P, v);
        else contract<T, 1, true>(a, b, w, P, v);
      } else {
        generic_contract<T, G, Q>(prov, a, b, P, v);
      }
#pragma unroll
      for (int i = 0; i < 24; ++i) acc[i] += v[i];
      if constexpr (G == 3) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            acc[24 + k * 4 + f] += xv[comb_rho(k)] * v[k * 4 + f];
            acc[48 + k * 4 + f] += xv[comb_sigma(k)] * v[k * 4 + f];
          }
      }
    }
    // warp sums, then the CTA's in FP64
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      T s = acc[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) red[warp][i] = (double)s;
    }
    __syncthreads();
    constexpr int NS = G == 3 ? 2 : 1;
    for (int e = threadIdx.x; e < NS * 64; e += blockDim.x) {
      int const slot = G + e / 64, idx = e % 64;
      int const r = idx / 16, s = (idx / 4) % 4, f = idx % 4;
      int i = -1;
      double sign = 1.0;
      if (slot < 4) {
        if (r < s) i = comb_index(r, s) * 4 + f;
      } else if (r < s) {
        i = 24 + comb_index(r, s) * 4 + f;
      } else if (r > s) {
        i = 48 + comb_index(s, r) * 4 + f;
        sign = -1.0;
      }
      double tot = 0.0;
      if (i >= 0)
        for (int q = 0; q < NW; ++q) tot += red[q][i];
      part[(((size_t)t * 5 + slot) * pstride + blockIdx.x) * 64 + idx] = sign * tot;
    }
    __syncthreads();
  }
}

// CTAs that wrote each slot's partials
struct SlotCtas {
  int n[5];
};

// out = the sum of the CTA partials of targets [0, n_t) of a chunk starting
// at target t0: raw ? out[(slot * n_y + t0 + t) * 64 + idx] : out[((t0 + t) * 5 + slot) * 64 + idx]
constexpr int kRedGroups = 8;  // threads per output element (CTA ranges)

__global__ void __launch_bounds__(64 * kRedGroups)
    p234_reduce_kernel(const double* __restrict__ part, int pstride, SlotCtas ncta, int n_y, int t0, int raw,
                       double* __restrict__ out) {
  int const t = blockIdx.x / 5, slot = blockIdx.x % 5, idx = threadIdx.x & 63, grp = threadIdx.x >> 6;
  const double* q = part + ((size_t)t * 5 + slot) * pstride * 64 + idx;
  double s = 0.0;
  for (int c = grp; c < ncta.n[slot]; c += kRedGroups) s += q[(size_t)c * 64];
  __shared__ double red[kRedGroups][64];
  red[grp][idx] = s;
  __syncthreads();
  if (grp != 0) return;
  s = 0.0;
  for (int g = 0; g < kRedGroups; ++g) s += red[g][idx];
  size_t const o = raw ? ((size_t)slot * n_y + t0 + t) * 64 + idx : (((size_t)t0 + t) * 5 + slot) * 64 + idx;
  out[o] = s;
}

}  // namespace p22

// ---- host side -------------------------------------------------------------
using namespace p22;

struct P22 {
  long long V = 0;
  double* d_pi = nullptr;   // site records [V][kRec] of double (FP32 uses half)
  double* d_part = nullptr;  // [kMaxTargets][5][grid_p234][64]
  double* d_p1part = nullptr;  // [sum of local extents][kP1Split][16]
  int grid_pi = 0;
  int grid_p234[2][4] = {};    // [FP64, FP32][G]: resident CTAs of each kernel
  int pstride = 0;             // the largest of them: the partials' CTA stride
};

namespace {

template <typename T, int G>
int grid_of(int nsm, int& grid) {
  int nb = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, p234_kernel<T, G, ClosedStandIn>,
                                                                kP234Threads, 0);
  if (e != cudaSuccess) return cuda_fail(e, "2+2 occupancy");
  if (nb < 1) return fail(HLBL_ECUDA, "2+2 kernel cannot be resident");
  grid = nsm * (nb < 8 ? nb : 8);
  return HLBL_OK;
}

}  // namespace

int p22_reserve(P22** st, const Geometry& geo, int nsm) {
  P22* s = *st;
  if (!s) {
    s = new P22();
    *st = s;
  }
  if (s->d_pi && s->V >= geo.V) return HLBL_OK;
  cudaFree(s->d_pi);
  cudaFree(s->d_part);
  cudaFree(s->d_p1part);
  s->d_pi = nullptr;
  s->d_part = nullptr;
  s->d_p1part = nullptr;
  s->V = 0;
  int rc = grid_of<double, 0>(nsm, s->grid_p234[0][0]);
  if (!rc) rc = grid_of<double, 1>(nsm, s->grid_p234[0][1]);
  if (!rc) rc = grid_of<double, 2>(nsm, s->grid_p234[0][2]);
  if (!rc) rc = grid_of<double, 3>(nsm, s->grid_p234[0][3]);
  if (!rc) rc = grid_of<float, 0>(nsm, s->grid_p234[1][0]);
  if (!rc) rc = grid_of<float, 1>(nsm, s->grid_p234[1][1]);
  if (!rc) rc = grid_of<float, 2>(nsm, s->grid_p234[1][2]);
  if (!rc) rc = grid_of<float, 3>(nsm, s->grid_p234[1][3]);
  if (rc) return rc;
  s->pstride = 0;
  for (auto& gp : s->grid_p234)
    for (int g : gp) s->pstride = g > s->pstride ? g : s->pstride;
  s->grid_pi = nsm * 8;
  cudaError_t e = cudaMalloc(&s->d_pi, (size_t)(geo.V > 0 ? geo.V : 1) * kRec * sizeof(double));
  if (e == cudaSuccess)
    e = cudaMalloc(&s->d_part, (size_t)kMaxTargets * 5 * s->pstride * 64 * sizeof(double));
  int const nslabs = geo.local[0] + geo.local[1] + geo.local[2] + geo.local[3];
  if (e == cudaSuccess) e = cudaMalloc(&s->d_p1part, (size_t)nslabs * kP1Split * 16 * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "2+2 work buffers");
  s->V = geo.V;
  return HLBL_OK;
}

void p22_destroy(P22* s) {
  if (!s) return;
  cudaFree(s->d_pi);
  cudaFree(s->d_part);
  cudaFree(s->d_p1part);
  delete s;
}

int p22_lmax(const Geometry& geo) {
  int l = geo.global[0];
  for (int r = 1; r < 4; ++r) l = geo.global[r] > l ? geo.global[r] : l;
  return l;
}

// The four per-target kernels of one chunk of targets; generic providers
// run every geometry on the partials' full CTA stride (their sums do not
// depend on the grid).
template <typename T, class Q>
static SlotCtas launch_p234(P22* s, cudaStream_t st, const P234Args& args, const Q& prov, const T* pi) {
  const int* gc = s->grid_p234[sizeof(T) == 4 ? 1 : 0];
  int g[4];
  for (int i = 0; i < 4; ++i) g[i] = std::is_same_v<Q, ClosedStandIn> ? gc[i] : s->pstride;
  p234_kernel<T, 0, Q><<<g[0], kP234Threads, 0, st>>>(args, prov, pi, s->pstride, s->d_part);
  p234_kernel<T, 1, Q><<<g[1], kP234Threads, 0, st>>>(args, prov, pi, s->pstride, s->d_part);
  p234_kernel<T, 2, Q><<<g[2], kP234Threads, 0, st>>>(args, prov, pi, s->pstride, s->d_part);
  p234_kernel<T, 3, Q><<<g[3], kP234Threads, 0, st>>>(args, prov, pi, s->pstride, s->d_part);
  return SlotCtas{{g[0], g[1], g[2], g[3], g[3]}};
}

template <typename T>
static void launch_all(P22* s, cudaStream_t st, const Geometry& geo, const P22Request& rq, P234Args& args,
                       const QedSel& q) {
  T* pi = reinterpret_cast<T*>(s->d_pi);
  int4 const gsw = make_int4(rq.gsw[0], rq.gsw[1], rq.gsw[2], rq.gsw[3]);
  long long const ntiles = (geo.V + kPiSites - 1) / kPiSites;
  int const gpi = (int)(ntiles < s->grid_pi ? ntiles : s->grid_pi);
  if (gpi > 0) {
    if constexpr (sizeof(T) == 4) {
      if (rq.x32) pi_kernel<float, true><<<gpi, kPiThreads, 0, st>>>(nullptr, rq.x32, geo, gsw, rq.iflavor, pi);
      else pi_kernel<float, false><<<gpi, kPiThreads, 0, st>>>(rq.fwd, nullptr, geo, gsw, rq.iflavor, pi);
    } else {
      pi_kernel<double, false><<<gpi, kPiThreads, 0, st>>>(rq.fwd, nullptr, geo, gsw, rq.iflavor, pi);
    }
  }
  int const lmax = p22_lmax(geo);
  int const nslabs = geo.local[0] + geo.local[1] + geo.local[2] + geo.local[3];
  p1_2p2_kernel<T><<<dim3(nslabs, kP1Split), kP1Threads, 0, st>>>(pi, geo, s->d_p1part);
  p1_2p2_finish_kernel<<<nslabs, 16, 0, st>>>(s->d_p1part, geo, gsw, lmax, rq.d_p1);
  for (int t0 = 0; t0 < rq.n_y; t0 += kMaxTargets) {
    int const nt = rq.n_y - t0 < kMaxTargets ? rq.n_y - t0 : kMaxTargets;
    args.n_t = nt;
    for (int t = 0; t < nt; ++t)
      for (int r = 0; r < 4; ++r)
        args.y[t][r] = mod_pos(rq.targets[4 * (t0 + t) + r] - rq.gsw[r], geo.global[r]);
    SlotCtas n;
    if (q.kind == kQedStandInClosed)
      n = launch_p234<T>(s, st, args, ClosedStandIn{}, pi);
    else
      n = with_provider(q, [&](auto prov) { return launch_p234<T>(s, st, args, prov, pi); });
    p234_reduce_kernel<<<nt * 5, 64 * kRedGroups, 0, st>>>(s->d_part, s->pstride, n, rq.n_y, t0, rq.raw_layout, rq.d_p234);
  }
}

int p22_run(P22** st, cudaStream_t stream, const Geometry& geo, const QedSel& q, int nsm,
            bool capturing, const P22Request& rq) {
  hlbl_qed_params const& qp = q.qp;
  if (!*st || (*st)->V < geo.V || !(*st)->d_pi) {
    if (capturing) return fail(HLBL_ESTATE, "2+2: work buffers not reserved before graph capture");
    if (int rc = p22_reserve(st, geo, nsm)) return rc;
  }
  P22* s = *st;
  int const lmax = p22_lmax(geo);
  cudaError_t e = cudaMemsetAsync(rq.d_p1, 0, (size_t)64 * lmax * sizeof(double), stream);
  if (e != cudaSuccess) return cuda_fail(e, "2+2 P1 clear");
  P234Args args{};
  args.geo = geo;
  for (int r = 0; r < 4; ++r) args.gsw[r] = rq.gsw[r];
  args.xunit = rq.xunit;
  args.qp = qp;
  args.r64f = (float)rq.r64;
  qed_f32_tables(qp, args.qf);
  if (rq.precision == HLBL_FP64) launch_all<double>(s, stream, geo, rq, args, q);
  else launch_all<float>(s, stream, geo, rq, args, q);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "2+2 launch");
  return HLBL_OK;
}

}  // namespace hg
