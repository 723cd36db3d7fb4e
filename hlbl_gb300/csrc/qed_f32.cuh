// qed_f32.cuh -- the stand-in QED weight (include/hlbl_gb300_qed.h) evaluated
// in FP32: the quadrature's per-node factors tabulated on the host
// (qed_f32_tables), the per-evaluation work on the device (weights_f32).
// Used by the FP32 kernel-sum path's weight kernel and by the FP32 2+2 pieces.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "hlbl_gb300_qed.h"

namespace hg {

// The stand-in QED weight's quadrature tabulated in FP32: per node u_i the
// factors of R_i^2 = uu X^2 + vv Y^2 + uv2 X Y c and g_i h_j(u_i); the
// exponents as powers of two, e2_j = -m_j log2(e).
struct QedF32 {
  float l2;
  float e2[HLBL_QED_NW];
  int geometric;            // m_j = m_0 + j dm for every j
  float de2;                // -dm log2(e)
  float dmneg;              // -dm
  float uu[HLBL_QED_NQ], vv[HLBL_QED_NQ], uv2[HLBL_QED_NQ];
  float wh[HLBL_QED_NQ][HLBL_QED_NW];
  float mneg[HLBL_QED_NW];  // -m_j
};


inline void qed_f32_tables(const hlbl_qed_params& qp, QedF32& q) {
  double const log2e = 1.4426950408889634;  // 1 / ln 2
  q.l2 = (float)(qp.lambda * qp.lambda);
  for (int j = 0; j < 6; ++j) {
    q.e2[j] = (float)(-qp.mass[j] * log2e);
    q.mneg[j] = (float)(-qp.mass[j]);
  }
  double const dm = qp.mass[1] - qp.mass[0];
  q.geometric = 1;
  for (int j = 2; j < 6; ++j)
    if (fabs(qp.mass[j] - (qp.mass[0] + j * dm)) > 1e-12 * fabs(qp.mass[j])) q.geometric = 0;
  q.de2 = (float)(-dm * log2e);
  q.dmneg = (float)(-dm);
  for (int i = 0; i < HLBL_QED_NQ; ++i) {
    double const u = qp.node[i], v = 1.0 - u;
    q.uu[i] = (float)(u * u);
    q.vv[i] = (float)(v * v);
    q.uv2[i] = (float)(-2.0 * u * v);
    double const h[6] = {1.0, u, v, u * v, u * u, v * v};
    for (int j = 0; j < 6; ++j) q.wh[i][j] = (float)(qp.weight[i] * h[j]);
  }
}


// The hardware approximations (PTX rcp/rsqrt/ex2 .approx.ftz): relative
// errors of a few 1e-7 on the ranges used here (1 + R^2 >= 1,
// R^2 + Lambda^2 >= Lambda^2 > 0, exponents <= 0 of moderate size).
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// The six stand-in weights in FP32: the FP64 definition's quadrature with
// the per-node factors tabulated in FP32 on the host. FAST: exp(-m_j r) as
// 2^(e2_j r) by the hardware ex2, rcp and rsqrt approximations (a few 1e-7
// per term), and with masses in arithmetic progression (m_j = m_0 + j dm, the
// stand-in's) exp(-m_0 r) g_i/(1+R^2) times powers of exp(-dm r): two
// operations per weight and node. Otherwise the correctly rounded FP32
// division and square root and expf (the kernel-sum path, whose chain total
// is held to 1e-6): with GEOM two expf per node and the powers of
// exp(-dm r) by five roundings to nearest (unbiased, a few 1e-7 at j = 5),
// else one expf per weight.
template <bool GEOM, bool FAST = true>
__device__ __forceinline__ void weights_f32(const QedF32& q, float X, float c, float Y, float w[6]) {
  float const X2 = X * X, Y2 = Y * Y, XYc = X * Y * c;
#pragma unroll
  for (int j = 0; j < 6; ++j) w[j] = 0.f;
  // fully unrolled: the node tables (kernel parameters) become immediate
  // constant operands instead of indexed constant loads
#pragma unroll
  for (int i = 0; i < HLBL_QED_NQ; ++i) {
    float r2 = fmaf(q.uu[i], X2, fmaf(q.vv[i], Y2, q.uv2[i] * XYc));
    r2 = fmaxf(r2, 0.f);
    if constexpr (FAST) {
      float const g = rcp_approx(1.f + r2);
      float const v = r2 + q.l2;
      float const r = v * rsqrt_approx(v);
      if constexpr (GEOM) {
        float te = g * ex2_approx(q.e2[0] * r);
        float const de = ex2_approx(q.de2 * r);
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          w[j] = fmaf(q.wh[i][j], te, w[j]);
          if (j < 5) te *= de;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 6; ++j) w[j] = fmaf(q.wh[i][j] * g, ex2_approx(q.e2[j] * r), w[j]);
      }
    } else {
      float const g = 1.f / (1.f + r2);
      float const r = sqrtf(r2 + q.l2);
      if constexpr (GEOM) {
        float te = g * expf(q.mneg[0] * r);
        float const de = expf(q.dmneg * r);
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          w[j] = fmaf(q.wh[i][j], te, w[j]);
          if (j < 5) te *= de;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 6; ++j) w[j] = fmaf(q.wh[i][j] * g, expf(q.mneg[j] * r), w[j]);
      }
    }
  }
}

// One node i of the FP64 quadrature (hlbl_qed_weights' loop body): adds its
// six terms into w. A warp evaluates a weight with one node per lane and a
// shuffle sum (qed_weights_fp64_warp).
__device__ __forceinline__ void qed_node_fp64(const hlbl_qed_params& p, int i, double X, double c, double Y,
                                              double w[HLBL_QED_NW]) {
  double const u = p.node[i], v = 1.0 - u;
  double r2 = u * u * X * X + v * v * Y * Y - 2.0 * u * v * X * Y * c;
  r2 = r2 > 0 ? r2 : 0.0;
  double const g = p.weight[i] / (1.0 + r2);
  double const r = sqrt(r2 + p.lambda * p.lambda);
  double const h[HLBL_QED_NW] = {1.0, u, v, u * v, u * u, v * v};
#pragma unroll
  for (int j = 0; j < HLBL_QED_NW; ++j) w[j] += g * h[j] * exp(-p.mass[j] * r);
}

// The FP64 weights of every lane in `mask` (each lane's own X, c, Y), the
// whole warp working on one lane's weight at a time: lane i < 16 takes node
// i, a shuffle tree sums the nodes, the owning lane keeps the six sums. Every
// lane of the warp calls it with the same mask.
__device__ __forceinline__ void qed_weights_fp64_warp(const hlbl_qed_params& p, unsigned mask, double X,
                                                      double c, double Y, double w[HLBL_QED_NW]) {
  static_assert(HLBL_QED_NQ <= 32, "one node per lane");
  int const lane = threadIdx.x & 31;
  while (mask) {
    int const src = __ffs(mask) - 1;
    mask &= mask - 1;
    double const Xs = __shfl_sync(0xffffffffu, X, src), cs = __shfl_sync(0xffffffffu, c, src),
                 Ys = __shfl_sync(0xffffffffu, Y, src);
    double t[HLBL_QED_NW];
#pragma unroll
    for (int j = 0; j < HLBL_QED_NW; ++j) t[j] = 0.0;
    if (lane < HLBL_QED_NQ) qed_node_fp64(p, lane, Xs, cs, Ys, t);
#pragma unroll
    for (int j = 0; j < HLBL_QED_NW; ++j) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t[j] += __shfl_xor_sync(0xffffffffu, t[j], o);
      if (lane == src) w[j] = t[j];
    }
  }
}

}  // namespace hg
