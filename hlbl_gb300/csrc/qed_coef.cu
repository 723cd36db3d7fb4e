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

int g_coef_grid = 0;

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
  constexpr int CS = coef_sites<P, T>();
  long long const vpad = F32 ? (geo.V + 31) / 32 * 32 : geo.V;
  long long const ntiles = (vpad + CS - 1) / CS;
  int const grid = (int)std::max<long long>(1, std::min<long long>(ntiles, std::max(1, g_coef_grid / npairs)));
  qed_coef_kernel<P, T, F32><<<dim3(grid, npairs), kCoefThreads, coef_smem<P, T>(), st>>>(geo, a, prov, out);
}

}  // namespace

int coef_init(int nsm) {
  g_coef_grid = nsm * 4;
  int rc = coef_attr<QedStandIn, double, false>();
  if (!rc) rc = coef_attr<QedStandIn, float, true>();
  if (!rc) rc = coef_attr<QedDense, double, false>();
  if (!rc) rc = coef_attr<QedDense, float, true>();
  if (!rc) rc = coef_attr<QedDenseKerv, double, false>();
  if (!rc) rc = coef_attr<QedDenseKerv, float, true>();
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
