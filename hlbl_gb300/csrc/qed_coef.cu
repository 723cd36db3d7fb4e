// qed_coef.cu -- the generic coefficient stage of pass 2: for every local
// site x of each pair, the 640 coefficients coef[mu][n] that fold the three
// QED kernel evaluations K(xm, ym), K(ym, xm), K(xm, x - y) and the zerohalf
// weights (ker_4pt_contraction, kernels/cuda_lattice.cu:403-476), from any
// provider (qed_provider.cuh). The contraction kernels then dot them with
// F[mu][n]; nothing downstream knows the tensor's structure.
//
// A CTA takes CS sites at a time: the sites' kernel arguments (xm, x - y,
// the zerohalf weights) into shared memory, one provider state per (site,
// evaluation), then every coefficient from three entries. Writes are
// ordered so that a warp stores contiguous runs of the output layout.
#include <cuda_runtime.h>

#include <algorithm>

#include "hlbl_gb300.h"
#include "hlbl_internal.h"
#include "qed_provider.cuh"

namespace hg {
namespace {

constexpr int kCoefThreads = 256;

template <class P, typename T>
constexpr int coef_sites() {
  // sites per CTA iteration: 32 (one FP32 tile) for small states; a
  // whole-tensor state (384 values per evaluation) takes 4
  return P::kState > 64 ? 4 : 32;
}
template <class P, typename T>
constexpr size_t coef_smem() {
  constexpr int CS = coef_sites<P, T>();
  return ((sizeof(T) * (size_t)CS * 3 * P::kState + 15) / 16) * 16 + sizeof(double) * CS * 12;
}

template <class P, typename T, bool F32>
__global__ void __launch_bounds__(kCoefThreads) qed_coef_kernel(Geometry geo, CoefArgs args, P prov,
                                                                T* __restrict__ out) {
  constexpr int CS = coef_sites<P, T>();
  constexpr int NS = P::kState;
  static_assert(!F32 || 32 % CS == 0, "an FP32 tile holds whole CTA site groups");
  extern __shared__ __align__(16) unsigned char smem[];
  T* s_st = reinterpret_cast<T*>(smem);  // [CS][3][NS]
  double* s_vec = reinterpret_cast<double*>(smem + ((sizeof(T) * (size_t)CS * 3 * NS + 15) / 16) * 16);  // [CS][12]
  int const t = threadIdx.x, pi = blockIdx.y;
  int const gsx[4] = {args.batch.p[pi].gsx[0], args.batch.p[pi].gsx[1], args.batch.p[pi].gsx[2],
                      args.batch.p[pi].gsx[3]};
  int const yv[4] = {args.batch.p[pi].yv[0], args.batch.p[pi].yv[1], args.batch.p[pi].yv[2],
                     args.batch.p[pi].yv[3]};
  double const xu = args.xunit;
  double ym[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ym[r] = coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]) * xu;
  out += (size_t)pi * args.stride;
  // the FP32 layout covers whole tiles of 32 sites (pads written as zeros)
  long long const vpad = F32 ? (geo.V + 31) / 32 * 32 : geo.V;
  long long const ntiles = (vpad + CS - 1) / CS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    long long const s0 = tile * CS;
    for (int it = t; it < CS * 4; it += kCoefThreads) {
      int const s = it >> 2, r = it & 3;
      int rel[4];
      rel_coords(geo, gsx, min(s0 + s, geo.V - 1), rel);
      s_vec[s * 12 + r] = coord_map(rel[r], geo.global[r]) * xu;
      s_vec[s * 12 + 4 + r] = coord_map_diff(rel[r], yv[r], geo.global[r]) * xu;
      s_vec[s * 12 + 8 + r] = (double)coord_map_zerohalf(rel[r], geo.global[r]);
    }
    __syncthreads();
    // one state per (site, evaluation): e = 0 K(xm, ym), 1 K(ym, xm), 2 K(xm, x - y)
    for (int it = t; it < CS * 3; it += kCoefThreads) {
      int const s = it / 3, e = it % 3;
      const double* xm = s_vec + s * 12;
      double a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        a[r] = e == 1 ? ym[r] : xm[r];
        b[r] = e == 0 ? ym[r] : (e == 1 ? xm[r] : xm[4 + r]);
      }
      prov.template prepare<T>(a, b, s_st + (size_t)it * NS);
    }
    __syncthreads();
    for (int it = t; it < CS * kCoefPerSite; it += kCoefThreads) {
      int s, mu, n;
      if constexpr (F32) {
        // consecutive threads: four n of a site, then the next site
        int const nl = it & 3, rest = it >> 2;
        s = rest % CS;
        int const g = rest / CS;  // (mu, n/4)
        mu = g / (kBtN / 4);
        n = (g % (kBtN / 4)) * 4 + nl;
      } else {
        s = it / kCoefPerSite;
        mu = (it / kBtN) & 3;
        n = it % kBtN;
      }
      long long const site = s0 + s;
      const T* st1 = s_st + (size_t)(s * 3) * NS;
      T v = T(0);
      if (site < geo.V) v = coef_value<P, T>(prov, st1, st1 + NS, st1 + 2 * NS, s_vec + s * 12 + 8, mu, n);
      if constexpr (F32) out[coef32_index(site, mu, n)] = v;
      else out[(size_t)site * kCoefPerSite + mu * kBtN + n] = v;
    }
    __syncthreads();
  }
}

// ---- providers linear in their state (QedDense) -----------------------------
// coef[mu][n] is then a fixed combination of table entries and the site's
// basis values: for j < 6,
//   sum_b (A[b][i1] phi_0[b] + A[b][i2] phi_1[b] - A[b][i3] phi_2[b]),
// and for j = 6 + tau, sum over the three pairs k touching tau of
//   (+zh_rho_k or -zh_sigma_k) sum_b A[b][i_k] phi_2[b].
// So each thread keeps the table columns of two adjacent outputs (n, n+1:
// the same j, lam and lam+1) in registers for the whole launch and walks the
// sites; the basis values of a site are the same for every thread (shared
// memory broadcast), and a packed FMA updates both outputs. Threads 0-191
// take the j < 6 outputs, 192-319 the zerohalf ones (uniform per warp).
// FP32 layout: a 32-site tile's outputs are staged in shared memory in the
// layout's order and written out contiguously.
constexpr int kLinThreads = 320;
constexpr int kLinNB = HLBL_QED_DENSE_NB;
constexpr int kLinSites = 32;
constexpr int kPhiPad = 16;
constexpr int kTileCoef = kLinSites * kCoefPerSite;  // 20,480 per FP32 tile

template <typename T>
__device__ __forceinline__ void dense_basis_t(const T a[4], const T b[4], T* phi) {
  T xx = T(0), yy = T(0), dd = T(0);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    T const d = a[r] - b[r];
    xx += a[r] * a[r];
    yy += b[r] * b[r];
    dd += d * d;
  }
  T const g = T(1) / (T(1) + xx + yy + T(0.5) * dd);
  phi[0] = g;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    phi[1 + r] = g * a[r];
    phi[5 + r] = g * b[r];
    phi[9 + r] = g * a[r] * b[r];
  }
#pragma unroll
  for (int r = kLinNB; r < kPhiPad; ++r) phi[r] = T(0);
}

template <typename T, bool F32>
__global__ void __launch_bounds__(kLinThreads, 1)
    qed_coef_linear_kernel(Geometry geo, CoefArgs args, const T* __restrict__ tab, T* __restrict__ out) {
  __shared__ __align__(16) T s_phi[kLinSites][3][kPhiPad];
  __shared__ T s_zh[kLinSites][4];
  extern __shared__ __align__(16) float s_stage[];  // F32: one tile's outputs
  int const t = threadIdx.x, pi = blockIdx.y;
  int const gsx[4] = {args.batch.p[pi].gsx[0], args.batch.p[pi].gsx[1], args.batch.p[pi].gsx[2],
                      args.batch.p[pi].gsx[3]};
  int const yv[4] = {args.batch.p[pi].yv[0], args.batch.p[pi].yv[1], args.batch.p[pi].yv[2],
                     args.batch.p[pi].yv[3]};
  T const xu = (T)args.xunit;
  out += (size_t)pi * args.stride;
  // this thread's outputs (mu, n) and (mu, n + 1)
  bool const zht = t >= 192;
  int const mu = zht ? (t - 192) / 32 : t / 48;
  int const n = zht ? 96 + 2 * ((t - 192) % 32) : 2 * (t % 48);
  int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
  // the three table columns of each output, as (n, n + 1) pairs; the
  // evaluation each column multiplies, and for zerohalf outputs the weight
  T tc[3][kLinNB][2];
  int ev[3], zi[3];
  T zs[3];
  if (!zht) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int const l = lam + h;
      int const ix[3] = {kerv_index(j, mu, nu, l), kerv_index(j, nu, mu, l), kerv_index(j, l, nu, mu)};
#pragma unroll
      for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int b = 0; b < kLinNB; ++b) tc[q][b][h] = (q == 2 ? -tab[b * HLBL_QED_NK + ix[q]] : tab[b * HLBL_QED_NK + ix[q]]);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) { ev[q] = q; zi[q] = 0; zs[q] = T(1); }
  } else {
    // the three pairs k = (r, g) that contain tau (every direction is in
    // exactly three), in k order
    int const tau = j - 6;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      int k = 0, c = 0;
#pragma unroll
      for (int kk = 0; kk < 6; ++kk) {
        bool const m = comb_rho(kk) == tau || comb_sigma(kk) == tau;
        if (m && c == q) k = kk;
        c += m ? 1 : 0;
      }
      int const r = comb_rho(k), g = comb_sigma(k);
      zi[q] = g == tau ? r : g;
      zs[q] = g == tau ? T(1) : T(-1);
      ev[q] = 2;
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int b = 0; b < kLinNB; ++b) tc[q][b][h] = tab[b * HLBL_QED_NK + kerv_index(k, lam + h, nu, mu)];
    }
  }
  long long const vpad = F32 ? (geo.V + kLinSites - 1) / kLinSites * kLinSites : geo.V;
  long long const ntiles = (vpad + kLinSites - 1) / kLinSites;
  T ym[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ym[r] = (T)coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]) * xu;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    long long const s0 = tile * kLinSites;
    if (t < kLinSites * 3) {
      int const s = t / 3, e = t % 3;
      int rel[4];
      rel_coords(geo, gsx, min(s0 + s, geo.V - 1), rel);
      T xm[4], xmy[4], a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        xm[r] = (T)coord_map(rel[r], geo.global[r]) * xu;
        xmy[r] = (T)coord_map_diff(rel[r], yv[r], geo.global[r]) * xu;
        a[r] = e == 1 ? ym[r] : xm[r];
        b[r] = e == 0 ? ym[r] : (e == 1 ? xm[r] : xmy[r]);
        if (e == 0) s_zh[s][r] = (T)coord_map_zerohalf(rel[r], geo.global[r]);
      }
      dense_basis_t<T>(a, b, &s_phi[s][e][0]);
    }
    __syncthreads();
    for (int s = 0; s < kLinSites; ++s) {
      long long const site = s0 + s;
      T v0 = T(0), v1 = T(0);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const T* ph = &s_phi[s][ev[q]][0];
        T a0 = T(0), a1 = T(0);
#pragma unroll
        for (int b = 0; b < kLinNB; ++b) {
          a0 = fma(tc[q][b][0], ph[b], a0);
          a1 = fma(tc[q][b][1], ph[b], a1);
        }
        T const w = zht ? zs[q] * s_zh[s][zi[q]] : T(1);
        v0 = fma(w, a0, v0);
        v1 = fma(w, a1, v1);
      }
      if (site >= geo.V) v0 = v1 = T(0);
      if constexpr (F32) {
        *reinterpret_cast<float2*>(s_stage + ((mu * (kBtN / 4) + (n >> 2)) * 32 + s) * 4 + (n & 3)) =
            make_float2((float)v0, (float)v1);
      } else {
        *reinterpret_cast<double2*>(out + (size_t)site * kCoefPerSite + mu * kBtN + n) = make_double2(v0, v1);
      }
    }
    __syncthreads();
    if constexpr (F32) {
      // the tile's block of the FP32 layout is contiguous
      float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(out) + (size_t)tile * kTileCoef);
      const float4* src = reinterpret_cast<const float4*>(s_stage);
      for (int i = t; i < kTileCoef / 4; i += kLinThreads) dst[i] = src[i];
      __syncthreads();
    }
  }
}

// The FP32 layout's version of the same stage: the table columns of the
// thread's two outputs are (n, n + 1) pairs and each basis value is stored
// twice, (phi, phi), so one packed FMA updates both outputs from one shared
// load; the code of each warp's output type has its evaluations fixed at
// compile time, and two sites go through each loop for more independent
// FMA chains.
__global__ void __launch_bounds__(kLinThreads, 1)
    qed_coef_linear32_kernel(Geometry geo, CoefArgs args, const float* __restrict__ tab,
                             float* __restrict__ out) {
  __shared__ __align__(16) float2 s_phi[kLinSites][3][kPhiPad];
  __shared__ float s_zh[kLinSites][4];
  extern __shared__ __align__(16) float s_stage[];  // one tile's outputs in the layout's order
  int const t = threadIdx.x, pi = blockIdx.y;
  int const gsx[4] = {args.batch.p[pi].gsx[0], args.batch.p[pi].gsx[1], args.batch.p[pi].gsx[2],
                      args.batch.p[pi].gsx[3]};
  int const yv[4] = {args.batch.p[pi].yv[0], args.batch.p[pi].yv[1], args.batch.p[pi].yv[2],
                     args.batch.p[pi].yv[3]};
  float const xu = (float)args.xunit;
  out += (size_t)pi * args.stride;
  bool const zht = t >= 192;  // warps 6-9: the zerohalf outputs (uniform per warp)
  int const mu = zht ? (t - 192) / 32 : t / 48;
  int const n = zht ? 96 + 2 * ((t - 192) % 32) : 2 * (t % 48);
  int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
  float2 tc[3][kLinNB];
  int zi[3];
  float zs[3];
  if (!zht) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      int const i0 = q == 0 ? kerv_index(j, mu, nu, lam) : q == 1 ? kerv_index(j, nu, mu, lam) : kerv_index(j, lam, nu, mu);
      int const i1 = q == 0 ? kerv_index(j, mu, nu, lam + 1)
                   : q == 1 ? kerv_index(j, nu, mu, lam + 1) : kerv_index(j, lam + 1, nu, mu);
      float const sg = q == 2 ? -1.f : 1.f;
#pragma unroll
      for (int b = 0; b < kLinNB; ++b)
        tc[q][b] = make_float2(sg * tab[b * HLBL_QED_NK + i0], sg * tab[b * HLBL_QED_NK + i1]);
      zi[q] = 0;
      zs[q] = 1.f;
    }
  } else {
    int const tau = j - 6;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      int k = 0, c = 0;
#pragma unroll
      for (int kk = 0; kk < 6; ++kk) {
        bool const m = comb_rho(kk) == tau || comb_sigma(kk) == tau;
        if (m && c == q) k = kk;
        c += m ? 1 : 0;
      }
      int const r = comb_rho(k), g = comb_sigma(k);
      zi[q] = g == tau ? r : g;
      zs[q] = g == tau ? 1.f : -1.f;
#pragma unroll
      for (int b = 0; b < kLinNB; ++b)
        tc[q][b] = make_float2(tab[b * HLBL_QED_NK + kerv_index(k, lam, nu, mu)],
                               tab[b * HLBL_QED_NK + kerv_index(k, lam + 1, nu, mu)]);
    }
  }
  long long const vpad = (geo.V + kLinSites - 1) / kLinSites * kLinSites;
  long long const ntiles = vpad / kLinSites;
  float ym[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ym[r] = (float)coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]) * xu;
  float* const st_base = s_stage + ((mu * (kBtN / 4) + (n >> 2)) * 32) * 4 + (n & 3);
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    long long const s0 = tile * kLinSites;
    if (t < kLinSites * 3) {
      int const s = t / 3, e = t % 3;
      int rel[4];
      rel_coords(geo, gsx, min(s0 + s, geo.V - 1), rel);
      float xm[4], xmy[4], a[4], b[4], phi[kPhiPad];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        xm[r] = (float)coord_map(rel[r], geo.global[r]) * xu;
        xmy[r] = (float)coord_map_diff(rel[r], yv[r], geo.global[r]) * xu;
        a[r] = e == 1 ? ym[r] : xm[r];
        b[r] = e == 0 ? ym[r] : (e == 1 ? xm[r] : xmy[r]);
        if (e == 0) s_zh[s][r] = (float)coord_map_zerohalf(rel[r], geo.global[r]);
      }
      dense_basis_t<float>(a, b, phi);
#pragma unroll
      for (int i = 0; i < kPhiPad; ++i) s_phi[s][e][i] = make_float2(phi[i], phi[i]);
    }
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < kLinSites; s += 2) {
      float2 v[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float2 acc[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const float2* ph = &s_phi[s + h][zht ? 2 : q][0];
          float2 a = make_float2(0.f, 0.f);
#pragma unroll
          for (int b = 0; b < kLinNB; ++b) a = __ffma2_rn(tc[q][b], ph[b], a);
          acc[q] = a;
        }
        if (zht) {
          v[h] = make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            float const w = zs[q] * s_zh[s + h][zi[q]];
            v[h] = __ffma2_rn(make_float2(w, w), acc[q], v[h]);
          }
        } else {
          v[h] = make_float2(acc[0].x + acc[1].x + acc[2].x, acc[0].y + acc[1].y + acc[2].y);
        }
        if (s0 + s + h >= geo.V) v[h] = make_float2(0.f, 0.f);
      }
      *reinterpret_cast<float2*>(st_base + s * 4) = v[0];
      *reinterpret_cast<float2*>(st_base + (s + 1) * 4) = v[1];
    }
    __syncthreads();
    // the tile's block of the FP32 layout is contiguous
    float4* dst = reinterpret_cast<float4*>(out + (size_t)tile * kTileCoef);
    const float4* src = reinterpret_cast<const float4*>(s_stage);
    for (int i = t; i < kTileCoef / 4; i += kLinThreads) dst[i] = src[i];
    __syncthreads();
  }
}

int g_coef_grid = 0;
int g_lin_grid = 0;

template <class P, typename T, bool F32>
int coef_attr() {
  constexpr size_t sm = coef_smem<P, T>();
  cudaError_t e = cudaFuncSetAttribute(qed_coef_kernel<P, T, F32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sm);
  if (e != cudaSuccess) return cuda_fail(e, "QED coefficient smem attribute");
  return HLBL_OK;
}

template <class P, typename T, bool F32>
void coef_run(const P& prov, const Geometry& geo, const CoefArgs& a, int npairs, T* out, cudaStream_t st) {
  if constexpr (IsLinear<P>::value) {
    long long const vpad = F32 ? (geo.V + kLinSites - 1) / kLinSites * kLinSites : geo.V;
    long long const ntiles = (vpad + kLinSites - 1) / kLinSites;
    int const grid = (int)std::max<long long>(1, std::min<long long>(ntiles, std::max(1, g_lin_grid / npairs)));
    if constexpr (F32) {
      qed_coef_linear32_kernel<<<dim3(grid, npairs), kLinThreads, kTileCoef * sizeof(float), st>>>(
          geo, a, prov.t32, out);
    } else {
      qed_coef_linear_kernel<T, F32><<<dim3(grid, npairs), kLinThreads, 0, st>>>(geo, a, prov.t64, out);
    }
    return;
  }
  constexpr int CS = coef_sites<P, T>();
  long long const vpad = F32 ? (geo.V + 31) / 32 * 32 : geo.V;
  long long const ntiles = (vpad + CS - 1) / CS;
  int const grid = (int)std::max<long long>(1, std::min<long long>(ntiles, std::max(1, g_coef_grid / npairs)));
  qed_coef_kernel<P, T, F32><<<dim3(grid, npairs), kCoefThreads, coef_smem<P, T>(), st>>>(geo, a, prov, out);
}

}  // namespace

int coef_init(int nsm) {
  g_coef_grid = nsm * 4;
  {
    cudaError_t e = cudaFuncSetAttribute(qed_coef_linear32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTileCoef * (int)sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "QED coefficient (linear) smem attribute");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, qed_coef_linear32_kernel, kLinThreads,
                                                      kTileCoef * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "QED coefficient (linear) occupancy");
    g_lin_grid = nsm * (nb > 0 ? nb : 1);
  }
  int rc = coef_attr<QedStandIn, double, false>();
  if (!rc) rc = coef_attr<QedStandIn, float, true>();
  if (!rc) rc = coef_attr<QedDense, double, false>();
  if (!rc) rc = coef_attr<QedDense, float, true>();
  if (!rc) rc = coef_attr<QedDenseKerv, double, false>();
  if (!rc) rc = coef_attr<QedDenseKerv, float, true>();
#ifdef HLBL_WITH_KQED
  if (!rc) rc = coef_attr<QedKqed, double, false>();
  if (!rc) rc = coef_attr<QedKqed, float, true>();
#endif
  return rc;
}

int coef_launch(const QedSel& q, bool f32, const Geometry& geo, const PairBatch& b, double xunit,
                void* out, cudaStream_t st) {
  CoefArgs a{};
  a.batch = b;
  a.xunit = xunit;
  a.stride = f32 ? coef32_per_pair(geo.V) : coef64_per_pair(geo.V);
  with_provider(q, [&](auto prov) {
    using P = decltype(prov);
    if (f32) coef_run<P, float, true>(prov, geo, a, b.n, static_cast<float*>(out), st);
    else coef_run<P, double, false>(prov, geo, a, b.n, static_cast<double*>(out), st);
    return 0;
  });
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "QED coefficient launch");
  return HLBL_OK;
}

}  // namespace hg
