// qed_provider.cuh -- the QED kernel as a pluggable provider, and the
// generic coefficient stage of pass 2.
//
// Pass 2 (ker_4pt_contraction, kernels/cuda_lattice.cu:277-484) weights each
// site x with three evaluations of KQED's QED_Mkernel_L2(0.4, a, b, temps,
// kerv[6][4][4][4]) (cuda_lattice.cu:266-275, calls at :435, :448, :461):
// e = 0: K(xm, ym), e = 1: K(ym, xm), e = 2: K(xm, x - y). The library folds
// the three tensors and the zerohalf weights into 640 coefficients per site,
//   coef[mu][(k, nu, lam)]   = K1[k][mu][nu][lam] + K2[k][nu][mu][lam] - K3[k][lam][nu][mu]
//   coef[mu][(6+t, nu, lam)] = sum_k K3[k][lam][nu][mu] (zh_rho_k [sigma_k = t] - zh_sigma_k [rho_k = t]),
// which the contraction dots with F[mu][n] = Re Tr(D_mu M_n).
//
// A provider gives any entry kerv[k][mu][nu][lam] of one evaluation K(a, b):
//   static constexpr int kState;                         values per evaluation
//   template <T> void prepare(const double a[4], const double b[4], T* st) const;
//   template <T> T entry(const T* st, int i) const;      i = ((k*4 + mu)*4 + nu)*4 + lam
// prepare runs once per (site, evaluation); entry as often as the
// contraction needs. Providers here:
//   QedStandIn   the stand-in of hlbl_gb300_qed.h: state (a, b, w[6]), each
//                entry from its Kronecker structure
//   QedDense     the dense test weight of hlbl_gb300_qed.h: state phi[13],
//                each entry a 13-term dot with its row of the seeded table
//   QedKerv<Fn>  any device function with QED_Mkernel_L2's shape,
//                Fn::operator()(const double a[4], const double b[4],
//                double kerv[6][4][4][4]): the state is the whole tensor
//                (384 values), entry(i) reads it. This is where a linked
//                KQED plugs in.
// The generic paths (qed_coef_kernel -> the contraction kernels' coefficient
// input; the generic 2+2 kernels) take any of them and use no structure of
// the tensor; the closed-form paths of the stand-in stay as its fast variant.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "contract_kernels.cuh"
#ifdef HLBL_WITH_KQED
#include "KQED.h"
#endif

namespace hg {

// The QED kernel a context weights with (hlbl_ctx_set_qed_kernel).
enum QedKind {
  kQedStandInClosed = 0,   // the stand-in through its closed-form paths
  kQedStandInGeneric = 1,  // the stand-in through the generic paths
  kQedDense = 2,           // the dense test weight, entry by entry
  kQedDenseKerv = 3,       // the dense test weight as a whole-tensor function
  kQedKqed = 4,            // a linked KQED's QED_Mkernel_L2 (builds with HLBL_WITH_KQED)
};
constexpr int kQedKinds = 5;

// entry index of kerv[k][mu][nu][lam]
__host__ __device__ constexpr int kerv_index(int k, int mu, int nu, int lam) {
  return ((k * 4 + mu) * 4 + nu) * 4 + lam;
}

struct QedStandIn {
  static constexpr int kState = 14;
  hlbl_qed_params qp;
  QedF32 qf;      // its FP32 quadrature tables (qed_f32.cuh)
  double r64;     // FP32 states: the FP64 weights where min(|a|, |b|) < r64
  template <typename T>
  __device__ __forceinline__ void prepare(const double a[4], const double b[4], T* st) const {
    double X, c, Y, w[HLBL_QED_NW];
    hlbl_qed_invariants(a, b, &X, &c, &Y);
    if (sizeof(T) == 4 && fmin(X, Y) >= r64) {
      // the FP32 path's weight, as the closed-form FP32 path evaluates it
      float wf[HLBL_QED_NW];
      if (qf.geometric) weights_f32<true, false>(qf, (float)X, (float)c, (float)Y, wf);
      else weights_f32<false, false>(qf, (float)X, (float)c, (float)Y, wf);
#pragma unroll
      for (int j = 0; j < HLBL_QED_NW; ++j) w[j] = wf[j];
    } else {
      hlbl_qed_weights(&qp, X, c, Y, w);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      st[r] = (T)a[r];
      st[4 + r] = (T)b[r];
    }
#pragma unroll
    for (int j = 0; j < HLBL_QED_NW; ++j) st[8 + j] = (T)w[j];
  }
  template <typename T>
  __device__ __forceinline__ T entry(const T* st, int i) const {
    return qed_entry_t<T>(st, i >> 6, (i >> 4) & 3, (i >> 2) & 3, i & 3);
  }
};

struct QedDense {
  static constexpr int kState = HLBL_QED_DENSE_NB;
  // every entry is linear in the state: entry(st, i) = sum_b table[b][i] st[b]
  // (qed_coef.cu's coefficient stage has a kernel for such providers)
  static constexpr bool kLinear = true;
  const double* t64;  // [13][384], device
  const float* t32;   // the same rounded to FP32
  template <typename T>
  __device__ __forceinline__ void prepare(const double a[4], const double b[4], T* st) const {
    double phi[HLBL_QED_DENSE_NB];
    hlbl_qed_dense_basis(a, b, phi);
#pragma unroll
    for (int j = 0; j < HLBL_QED_DENSE_NB; ++j) st[j] = (T)phi[j];
  }
  template <typename T>
  __device__ __forceinline__ T entry(const T* st, int i) const {
    const T* tab;
    if constexpr (sizeof(T) == 8) tab = reinterpret_cast<const T*>(t64);
    else tab = reinterpret_cast<const T*>(t32);
    T v = T(0);
#pragma unroll
    for (int b = 0; b < HLBL_QED_DENSE_NB; ++b) v = fma(__ldg(tab + b * HLBL_QED_NK + i), st[b], v);
    return v;
  }
};

template <class Fn>
struct QedKerv {
  static constexpr int kState = HLBL_QED_NK;
  Fn fn;
  template <typename T>
  __device__ __forceinline__ void prepare(const double a[4], const double b[4], T* st) const {
    if constexpr (sizeof(T) == 8) {
      fn(a, b, reinterpret_cast<double(*)[4][4][4]>(st));
    } else {
      double kv[6][4][4][4];
      fn(a, b, kv);
      const double* k = &kv[0][0][0][0];
      for (int i = 0; i < HLBL_QED_NK; ++i) st[i] = (T)k[i];
    }
  }
  template <typename T>
  __device__ __forceinline__ T entry(const T* st, int i) const {
    return st[i];
  }
};

// The dense test weight as a function of QED_Mkernel_L2's shape.
struct DenseKervFn {
  const double* t64;
  __device__ __forceinline__ void operator()(const double a[4], const double b[4],
                                             double kerv[6][4][4][4]) const {
    hlbl_qed_dense_kernel(t64, a, b, kerv);
  }
};
using QedDenseKerv = QedKerv<DenseKervFn>;

#ifdef HLBL_WITH_KQED
// KQED's own device function (kernels/cuda_lattice.cu:266-275 calls it as
// QED_Mkernel_L2(0.4, xm, ym, kqed_t, kerv)), linked from libKQED_cuda.a in a
// relocatable-device-code build; the temps travel by value, as the
// reference passes them to its kernels (cuda_lattice.cu:816-839).
struct KqedFn {
  QED_kernel_temps t;
  double lambda;
  __device__ __forceinline__ void operator()(const double a[4], const double b[4],
                                             double kerv[6][4][4][4]) const {
    QED_Mkernel_L2(lambda, a, b, t, kerv);
  }
};
using QedKqed = QedKerv<KqedFn>;
#endif

// What a context passes down: the kind and everything its providers need.
struct QedSel {
  int kind = kQedStandInClosed;
  hlbl_qed_params qp{};
  QedF32 qf{};
  double r64 = 0.0;
  const double* t64 = nullptr;
  const float* t32 = nullptr;
#ifdef HLBL_WITH_KQED
  QED_kernel_temps kq{};
#endif
};

// Host: call f(provider) with the provider of a generic kind.
template <class F>
decltype(auto) with_provider(const QedSel& q, F&& f) {
  if (q.kind == kQedDense) return f(QedDense{q.t64, q.t32});
  if (q.kind == kQedDenseKerv) return f(QedDenseKerv{DenseKervFn{q.t64}});
#ifdef HLBL_WITH_KQED
  if (q.kind == kQedKqed) return f(QedKqed{KqedFn{q.kq, q.qp.lambda}});
#endif
  return f(QedStandIn{q.qp, q.qf, q.r64});
}

template <class P, class = void>
struct IsLinear : std::false_type {};
template <class P>
struct IsLinear<P, std::void_t<decltype(P::kLinear)>> : std::bool_constant<P::kLinear> {};

// One coefficient of a site from its three evaluations' states.
template <class P, typename T>
__device__ __forceinline__ T coef_value(const P& prov, const T* st1, const T* st2, const T* st3,
                                        const double* zh, int mu, int n) {
  int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
  if (j < 6)
    return prov.template entry<T>(st1, kerv_index(j, mu, nu, lam)) +
           prov.template entry<T>(st2, kerv_index(j, nu, mu, lam)) -
           prov.template entry<T>(st3, kerv_index(j, lam, nu, mu));
  int const tau = j - 6;
  T cf = T(0);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    int const r = comb_rho(k), g = comb_sigma(k);
    if (g == tau) cf += (T)zh[r] * prov.template entry<T>(st3, kerv_index(k, lam, nu, mu));
    if (r == tau) cf -= (T)zh[g] * prov.template entry<T>(st3, kerv_index(k, lam, nu, mu));
  }
  return cf;
}

struct CoefArgs {
  PairBatch batch;   // gsx, yv of each pair (blockIdx.y)
  double xunit;
  size_t stride;     // elements per pair in the output
};

// Launch the coefficient stage for b.n pairs: FP64 layout (f32 = false,
// T = double) or FP32 layout (f32 = true, T = float). qed_coef.cu.
int coef_init(int nsm);
int coef_launch(const QedSel& q, bool f32, const Geometry& geo, const PairBatch& b, double xunit,
                void* out, cudaStream_t st);

}  // namespace hg
