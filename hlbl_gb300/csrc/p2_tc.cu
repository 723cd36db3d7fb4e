// p2_tc.cu -- pass 2 of the mixed-precision path on the 5th-generation tensor
// cores (tcgen05), the same sum as p2_kernel<float, 2, TS>:
//   F[mu][n] = sum_k Dr_mu[k] Bt[k][n],  dtmp = -sum_{mu,n} coef[mu][n] F[mu][n]
// (ker_4pt_contraction, cuda_lattice.cu:277-484, restructured as in
// contract_kernels.cuh).
//
// Per CTA (one per SM, persistent over tiles of 32 sites) and per phase
// (tile, flavour f): the 128 x 160 product F = A . B^T, A = Dr with rows
// (mu, site) = mu*32 + site and K = 288 = (p, q, re/im), B = Bt^T. Products
// are FP32 in the 3xTF32 form A_hi B_hi + A_hi B_lo + A_lo B_hi (hi = the
// TF32 rounding, lo = the TF32 rounding of the rest), accumulated in TMEM.
//
// Warp roles (15 warps):
//   0      TMA producer of the FP32 input rows (S = x[1-f] rows q, Y = y[f]
//          rows p: 3 KB per (flavour, ia, tile)) -- one thread
//   1      TMA producer of the B chunks (16 k x 160 n, hi and lo, 20 KB) -- one thread
//   2      TMEM allocation; tcgen05.mma issue and commits -- one thread
//   3-10   D formation, two groups of four warps on alternate chunks of
//          16 k (8 (p, q): half of a block of 4 p x 4 q): warp j of a group
//          forms the chunk's j-th pair of (p, q) (one Y row, two S rows) for
//          its lane's site: O = Y conj(S) spin blocks -> D_mu -> hi/lo ->
//          shared memory in the K-major no-swizzle core-matrix layout
//   11-14  epilogue: one TMEM lane quadrant each (warp % 4 = mu); per phase,
//          the F rows from TMEM dotted with the QED coefficients of the
//          row's site, into a compensated FP64 sum
// The tensor cores accumulate in FP32 with truncation (biased toward zero),
// so the error grows with the number of MMAs added into one accumulator and
// the small hi.lo and lo.hi products lose most of their bits if added into
// the large hi.hi sum. Three accumulators of 160 TMEM columns: the
// corrections go to their own, and the hi.hi sum of chunks 0-8 and of
// chunks 9-17 to the two main buffers; the epilogue adds the second half
// and the corrections into the first (FP32, round-to-nearest) before the
// dot. The two main buffers swap roles every phase: the next phase's first
// half only waits for that fold, its second half for the dot.
// Pipelines (mbarriers; every wait bounded, kWaitLimit polls):
//   rows -> D warps (S rows of a block in a ring of 2 blocks, Y rows of a
//   p-block by halves in a ring of 3),
//   D warps -> MMA (A ring of 5), B producer -> MMA (B ring of 5), one
//   commit per chunk frees both stages,
//   MMA -> epilogue (acc_full), epilogue -> MMA (folded, dotted).
//
// Inputs are the FP32 tile copies pass 1 writes while it converts each
// block (x32/y32: [f][ia][tile][2][6][16][4] floats, f32_tile_off: a site's
// 24 components as six 16-byte groups, 32 sites per tile in two halves), so
// pass 2 reads half the bytes of the FP64 blocks and converts nothing.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "contract_kernels.cuh"
#include "hlbl_gb300.h"
#include "hlbl_internal.h"
#include "p2_tc.h"

namespace hg {
namespace tc {

constexpr int kSites = 32;                 // sites per tile
constexpr int kM = 128;                    // MMA rows: (mu, site)
constexpr int kKc = 16;                    // K per chunk
constexpr int kChunks = kBtK / kKc;        // 18
// A and B rings of the same depth (OpT::kStages: 5 for TF32 operands, 10 for
// FP16), released by one commit per chunk: the tensor pipe's completion
// reaches the waiting producers about 2,500 cycles after a chunk is issued, so
// several chunks must be in flight to keep it busy; one commit per chunk frees
// the A and the B stage (a deeper ring for one of them with a second commit
// per chunk measured slower).
// K order: blocks of 4 p x 4 q (two chunks each), q-blocks inner, so both row
// sets stream through small rings instead of one being held for a whole
// phase: the S rows 4 bq..4 bq+3 of a block (a ring of two blocks; fetched
// again, from L2, for each p-block) and the Y rows of a p-block by halves,
// half h (rows 4 bp + 2h, 4 bp + 2h + 1) read only by D group h (a ring of
// three halves). This leaves room for five A and B stages.
constexpr int kRowsPerGroup = 4, kBlocksQ = 3;
constexpr int kYRows = 2;
constexpr int kBlocks = 9;  // per phase: 3 p-blocks x 3 q-blocks
constexpr int kHalf = kChunks / 2;               // chunks per main-accumulator half
constexpr uint32_t kCorrCol = 2 * kBtN;          // the correction accumulator's first column
constexpr int kAPart = kM * kKc;           // floats per A part (hi or lo)
constexpr int kBPart = kBtN * kKc;         // floats per B part
constexpr int kWarpRows = 0, kWarpB = 1, kWarpMma = 2, kWarpD0 = 3, kDWarps = 8;
constexpr int kDGroup = 4;  // D warps per chunk (a group); kDWarps / kDGroup chunks in flight
constexpr int kWarpE0 = kWarpD0 + kDWarps, kEWarps = 4;
constexpr int kThreads = 32 * (kWarpE0 + kEWarps);
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kRowBytes = kRowF32 * 4;  // 3072

// Operand type of the products (both TF32 or both FP16; D is F32 either way).
// FP16: the same 3-term split as TF32 (hi = the rounding of the value, lo =
// the rounding of the rest: 11 + 11 significant bits) in half the bytes, with
// one MMA of K = 16 per product and chunk instead of two of K = 8, so the
// rings hold twice the chunks. FP16's exponent range is met by power-of-two
// scales: A by 2^(15 - e) with 2^e above the bound 24 max|Y| max|S| of every
// D value (from the per-flavour maxima the tile copies carry), B by the same
// rule from max|Bt| per pair and flavour; the epilogue divides each row's dot
// by the product (exact). The bytes saved go to deeper row rings (four S
// blocks, six Y halves instead of two and three), which the D warps were
// waiting on, and to seven operand stages.
template <bool F16> struct OpT;
// kSGroups, kYSlots: depths of the S-block and Y-half rings
// kBParts: B as hi + lo (TF32) or hi + lo + lo2 (FP16, split from the FP64
// value: ~33 significant bits, as B's rounding error would repeat at every
// site of a pair)
template <> struct OpT<false> {
  static constexpr int kStages = 5, kElem = 4, kSGroups = 2, kYSlots = 3, kBParts = 2;
  static constexpr uint32_t kFmt = 2;  // TF32
};
template <> struct OpT<true> {
  static constexpr int kStages = 6, kElem = 2, kSGroups = 4, kYSlots = 6, kBParts = 3;
  static constexpr uint32_t kFmt = 0;  // F16
};
// instruction descriptor: D F32, A and B of the operand type, both K-major,
// N = 160, M = 128
template <bool F16>
constexpr uint32_t idesc() {
  return (1u << 4) | (OpT<F16>::kFmt << 7) | (OpT<F16>::kFmt << 10) | ((uint32_t)(kBtN >> 3) << 17) |
         ((uint32_t)(kM >> 4) << 24);
}
constexpr uint32_t kIdesc = idesc<false>();

template <bool F16>
struct __align__(1024) SmemT {
  static constexpr int kSt = OpT<F16>::kStages;
  static constexpr int kAPartB = kAPart * OpT<F16>::kElem, kBPartB = kBPart * OpT<F16>::kElem;  // bytes
  static constexpr int kSGroups = OpT<F16>::kSGroups, kYSlots = OpT<F16>::kYSlots;
  float S[kSGroups][kRowsPerGroup][kRowF32];
  float Y[kYSlots][kYRows][kRowF32];
  __align__(16) unsigned char A[kSt][2][kAPartB];
  __align__(16) unsigned char B[kSt][OpT<F16>::kBParts][kBPartB];
  uint64_t s_full[kSGroups], s_empty[kSGroups], y_full[kYSlots], y_empty[kYSlots];
  uint64_t a_full[kSt], b_full[kSt], a_empty[kSt], b_empty[kSt];
  uint64_t acc_full, folded, dotted, mma_done;
  uint32_t taddr;
  int fail;
  double red[kEWarps][2][2];
};
using Smem = SmemT<false>;
static_assert(sizeof(SmemT<false>) <= 232448 && sizeof(SmemT<true>) <= 232448,
              "pass-2 shared memory above the 227 KB a CTA may have");

// FP16 hi and lo parts of two values, packed as the MMA reads them (the first
// value in the low half)
__device__ __forceinline__ void f16_split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  __half2 const h = __floats2half2_rn(a, b);
  float2 const f = __half22float2(h);
  __half2 const l = __floats2half2_rn(a - f.x, b - f.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}
// 2^(15 - e) for the smallest e with bound < 2^e: scales values bounded by
// `bound` into FP16's range with a factor of two to spare (1 for bound 0)
__host__ __device__ __forceinline__ float f16_scale(float bound) {
  if (!(bound > 0.f) || !(bound <= 3.0e38f)) return 1.f;  // zero, NaN or infinite inputs
  int e;
  frexpf(bound, &e);  // bound = m 2^e, m in [0.5, 1)
  int const k = 15 - e;
  return ldexpf(1.f, k < -126 ? -126 : (k > 127 ? 127 : k));
}

// ---- tcgen05 / TMA helpers ---------------------------------------------------
// shared-memory matrix descriptor, no swizzle: start, leading byte offset
// (between core matrices along K), stride byte offset (between 8-row groups)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// The same rounding (to nearest, ties away from zero, the low 13 bits
// cleared) on the integer pipe, for finite x: adding half a TF32 unit to the
// magnitude bits carries into the kept bits exactly when the dropped part is
// at least half; a carry into the exponent is the correct round-up. The
// D-formation warps round 16 values per (p, q) pair this way.
__device__ __forceinline__ float tf32_round(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}
__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc<true>()), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t addr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(addr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_st16(uint32_t addr, const float v[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(addr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// A wait that gives up when the CTA has failed or after kWaitLimit polls
// (then it marks the CTA failed). Returns false on give-up.
__device__ __forceinline__ bool wait_or_fail(uint64_t* bar, uint32_t parity, volatile int* fail) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 63 && *fail) return false;
  }
  *fail = 1;
  return false;
}

// ---- the QED-weighted dot of one row (mu = MU, fixed) ------------------------------
// The row's contribution is sum_n coef[MU][n] F[n] with n = (j, nu, lam),
// coef[MU][(k, nu, lam)] = E1(k, MU, nu, lam) + E2(k, nu, MU, lam) - E3(k, lam, nu, MU)
// (k < 6) and coef[MU][(6 + tau, nu, lam)] = sum_k c_k(tau) E3(k, lam, nu, MU)
// with c_k(tau) = [sigma_k = tau] zh_rho_k - [rho_k = tau] zh_sigma_k, where
// Ee(k, a, b, c) = kerv[k][a][b][c] of the stand-in tensor at the argument
// pair e: (xm, ym), (ym, xm), (xm, x - y) (hlbl_qed_entry: six terms w_0..w_5,
// each a Kronecker structure times coordinates). For fixed k the columns of
// F form a 4 x 4 matrix G[nu][lam], and each term's sum over (nu, lam)
// reduces to rows G.v, columns u.G, forms u.G.v, the trace and the
// antisymmetric part G[r][s] - G[s][r]; the sums below are those reductions.
struct SiteQ {
  float xm[4], ym[4], xmy[4], zh[4];
  float w[3][HLBL_QED_NW];
};

__device__ __forceinline__ float row_dot(const float* G, int i, const float* v) {
  return fmaf(G[4 * i + 3], v[3], fmaf(G[4 * i + 2], v[2], fmaf(G[4 * i + 1], v[1], G[4 * i] * v[0])));
}
__device__ __forceinline__ float col_dot(const float* G, int i, const float* u) {
  return fmaf(u[3], G[12 + i], fmaf(u[2], G[8 + i], fmaf(u[1], G[4 + i], u[0] * G[i])));
}

// sum_{nu,lam} E3(k, lam, nu, MU) G[nu][lam]; gx = G.xm, gz = G.xmy (rows),
// zg = xmy.G (columns), xGx = xm.G.xm, tr = trace(G)
template <int MU, int K>
__device__ __forceinline__ float d3(const float* G, const SiteQ& q, const float* gx, const float* gz,
                                    const float* zg, float xGx, float tr) {
  constexpr int r = comb_rho(K), s = comb_sigma(K);
  const float* x = q.xm;
  const float* y = q.xmy;
  const float* w = q.w[2];
  float const anti = G[4 * r + s] - G[4 * s + r];
  float v = -w[0] * x[MU] * anti;
  v = fmaf(w[3] * (x[r] * y[s] - x[s] * y[r]) * (x[MU] + y[MU]), tr, v);
  v = fmaf(w[4] * y[MU], x[r] * zg[s] - x[s] * zg[r], v);
  if constexpr (MU == s) v += w[1] * zg[r] + w[2] * (gx[r] - gz[r]) + w[5] * y[r] * xGx;
  if constexpr (MU == r) v -= w[1] * zg[s] + w[2] * (gx[s] - gz[s]) + w[5] * y[s] * xGx;
  return v;
}

// j = K < 6: E1 + E2 - E3 against G = F[(K, ., .)]
template <int MU, int K>
__device__ __forceinline__ float dot_k(const float* G, const SiteQ& q) {
  constexpr int r = comb_rho(K), s = comb_sigma(K);
  const float* xm = q.xm;
  const float* ym = q.ym;
  const float* xmy = q.xmy;
  float gx[4], gy[4], gz[4], zg[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    gx[i] = row_dot(G, i, xm);
    gy[i] = row_dot(G, i, ym);
  }
  gz[r] = row_dot(G, r, xmy); gz[s] = row_dot(G, s, xmy);
  zg[r] = col_dot(G, r, xmy); zg[s] = col_dot(G, s, xmy);
  float const ygr = col_dot(G, r, ym), ygs = col_dot(G, s, ym);  // ym.G
  float const xgr = col_dot(G, r, xm), xgs = col_dot(G, s, xm);  // xm.G
  float const yGy = fmaf(ym[3], gy[3], fmaf(ym[2], gy[2], fmaf(ym[1], gy[1], ym[0] * gy[0])));
  float const xGx = fmaf(xm[3], gx[3], fmaf(xm[2], gx[2], fmaf(xm[1], gx[1], xm[0] * gx[0])));
  float const tr = G[0] + G[5] + G[10] + G[15];
  float const anti = G[4 * r + s] - G[4 * s + r];
  const float* w1 = q.w[0];
  const float* w2 = q.w[1];
  // E1: (a, b, c) = (MU, nu, lam) at (xm, ym)
  float v = w1[2] * (xm[MU] - ym[MU]) * anti;
  v = fmaf(w1[3] * (xm[r] * ym[s] - xm[s] * ym[r]), gx[MU] + gy[MU], v);
  v = fmaf(w1[5] * xm[MU], ym[r] * xgs - ym[s] * xgr, v);
  if constexpr (MU == r) v += w1[0] * gx[s] + w1[1] * ygs - w1[4] * xm[s] * yGy;
  if constexpr (MU == s) v += -w1[0] * gx[r] - w1[1] * ygr + w1[4] * xm[r] * yGy;
  // E2: (a, b, c) = (nu, MU, lam) at (ym, xm)
  v = fmaf(w2[1] * xm[MU], anti, v);
  v = fmaf(w2[3] * (ym[r] * xm[s] - ym[s] * xm[r]), gy[MU] + gx[MU], v);
  v = fmaf(w2[4] * xm[MU], ym[r] * gx[s] - ym[s] * gx[r], v);
  v = fmaf(w2[5] * ym[MU], xm[r] * ygs - xm[s] * ygr, v);
  if constexpr (MU == s) v += w2[0] * gy[r] - w2[2] * (ygr - xgr);
  if constexpr (MU == r) v += -w2[0] * gy[s] + w2[2] * (ygs - xgs);
  // - E3: (a, b, c) = (lam, nu, MU) at (xm, x - y)
  return v - d3<MU, K>(G, q, gx, gz, zg, xGx, tr);
}

// j = 6 + TAU: sum_k c_k(TAU) E3(k, lam, nu, MU) against G = F[(6 + TAU, ., .)]
template <int MU, int TAU>
__device__ __forceinline__ float dot_zh(const float* G, const SiteQ& q) {
  float gx[4], gz[4], zg[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    gx[i] = row_dot(G, i, q.xm);
    gz[i] = row_dot(G, i, q.xmy);
    zg[i] = col_dot(G, i, q.xmy);
  }
  const float* xm = q.xm;
  float const xGx = fmaf(xm[3], gx[3], fmaf(xm[2], gx[2], fmaf(xm[1], gx[1], xm[0] * gx[0])));
  float const tr = G[0] + G[5] + G[10] + G[15];
  float v = 0.f;
  auto term = [&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int r = comb_rho(k), g = comb_sigma(k);
    if constexpr (g == TAU || r == TAU) {
      float const e = d3<MU, k>(G, q, gx, gz, zg, xGx, tr);
      if constexpr (g == TAU) v = fmaf(q.zh[r], e, v);
      if constexpr (r == TAU) v = fmaf(-q.zh[g], e, v);
    }
  };
  term(std::integral_constant<int, 0>{});
  term(std::integral_constant<int, 1>{});
  term(std::integral_constant<int, 2>{});
  term(std::integral_constant<int, 3>{});
  term(std::integral_constant<int, 4>{});
  term(std::integral_constant<int, 5>{});
  return v;
}

// One phase's row: sum_n coef[MU][n] F[n], F at column c of this warp's lane
// quadrant (16 columns = one 4 x 4 matrix per j).
template <int MU>
__device__ __forceinline__ float epilogue_row(uint32_t lane_addr, uint32_t c, const SiteQ& q) {
  float f[16], a = 0.f;
#define HG_TC_K(J)                      \
  tmem_ld16(lane_addr + c + 16 * J, f); \
  tmem_wait_ld();                       \
  a += dot_k<MU, J>(f, q);
#define HG_TC_T(J)                      \
  tmem_ld16(lane_addr + c + 16 * J, f); \
  tmem_wait_ld();                       \
  a += dot_zh<MU, J - 6>(f, q);
  HG_TC_K(0) HG_TC_K(1) HG_TC_K(2) HG_TC_K(3) HG_TC_K(4) HG_TC_K(5)
  HG_TC_T(6) HG_TC_T(7) HG_TC_T(8) HG_TC_T(9)
#undef HG_TC_K
#undef HG_TC_T
  return a;
}

// Generic QED path: one phase's row dotted with the row's coefficients,
// read from the FP32 coefficient layout (crow: this row's (tile, mu, site)
// base; group g of four n at crow + g*128), one 16-column block of F per j.
// The next block's coefficients are loaded while the current one is dotted.
__device__ __forceinline__ float epilogue_row_generic(uint32_t lane_addr, uint32_t c, const float* crow) {
  float f[16], a = 0.f;
  float4 cf[4], cn[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) cf[i] = __ldg(reinterpret_cast<const float4*>(crow + i * 128));
#pragma unroll 1
  for (int jj = 0; jj < 10; ++jj) {
    if (jj + 1 < 10) {
#pragma unroll
      for (int i = 0; i < 4; ++i) cn[i] = __ldg(reinterpret_cast<const float4*>(crow + ((jj + 1) * 4 + i) * 128));
    }
    tmem_ld16(lane_addr + c + 16 * jj, f);
    tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      a = fmaf(cf[i].x, f[4 * i], a);
      a = fmaf(cf[i].y, f[4 * i + 1], a);
      a = fmaf(cf[i].z, f[4 * i + 2], a);
      a = fmaf(cf[i].w, f[4 * i + 3], a);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) cf[i] = cn[i];
  }
  return a;
}

// The D formation's closed forms of D_mu from the spin-block products follow
// from these phases (i^((2 - g5g_ph(mu, s1)) & 3) for s1 = 0..3).
constexpr int d_ph(int mu, int s1) { return (6 - g5g_ph(mu, s1)) & 3; }
static_assert(d_ph(0, 0) == 0 && d_ph(0, 1) == 0 && d_ph(0, 2) == 2 && d_ph(0, 3) == 2, "D_0 = a0 + a1 - a2 - a3");
static_assert(d_ph(3, 0) == 3 && d_ph(3, 1) == 1 && d_ph(3, 2) == 3 && d_ph(3, 3) == 1, "D_3 = i (a1 + a3 - a0 - a2)");
static_assert(d_ph(1, 0) == 3 && d_ph(1, 1) == 3 && d_ph(1, 2) == 3 && d_ph(1, 3) == 3, "D_1 = -i (b0 + b1 + b2 + b3)");
static_assert(d_ph(2, 0) == 0 && d_ph(2, 1) == 2 && d_ph(2, 2) == 0 && d_ph(2, 3) == 2, "D_2 = b0 - b1 + b2 - b3");

// ---- the kernel ------------------------------------------------------------------
// kGeneric: the QED weighting from the coefficient tensor of args.coef (any
// QED kernel, qed_provider.cuh) instead of the stand-in's closed form.
// kF16: FP16 operands (OpT<true>); btu then holds FP16 parts and bscale the
// B scale per (pair, flavour).
template <bool kGeneric, bool kF16>
__global__ void __launch_bounds__(kThreads, 1)
p2tc_kernel(TcBatch tb, Geometry geo, P2Args args, const void* __restrict__ btu,
            const float* __restrict__ bscale, double* __restrict__ partials, int* __restrict__ err) {
  using Sm = SmemT<kF16>;
  constexpr int kSt = Sm::kSt, kSGroups = Sm::kSGroups, kYSlots = Sm::kYSlots;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  Sm& sm = *reinterpret_cast<Sm*>(smem_raw);
  volatile int* fail = &sm.fail;
  int const t = threadIdx.x, warp = t >> 5, lane = t & 31;
  int const pi = blockIdx.y;
  long long const ntiles = (geo.V + kSites - 1) / kSites;
  long long const my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  int const nph = (int)(2 * my_tiles);
  const float* __restrict__ x32 = tb.x32[pi];
  const float* __restrict__ y32 = tb.y32;
  auto row_ptr = [&](const float* base, int f, int ia, long long tile) {
    return base + ((size_t)(f * 12 + ia) * ntiles + tile) * kRowF32;
  };

  if (t == 0) {
    for (int i = 0; i < kSGroups; ++i) { mbar_init(&sm.s_full[i], 1); mbar_init(&sm.s_empty[i], kDWarps); }
    for (int i = 0; i < kYSlots; ++i) { mbar_init(&sm.y_full[i], 1); mbar_init(&sm.y_empty[i], kDGroup); }
    for (int i = 0; i < kSt; ++i) { mbar_init(&sm.a_full[i], kDGroup); mbar_init(&sm.a_empty[i], 1); }
    for (int i = 0; i < kSt; ++i) { mbar_init(&sm.b_full[i], 1); mbar_init(&sm.b_empty[i], 1); }
    mbar_init(&sm.acc_full, 1);
    mbar_init(&sm.folded, kEWarps);
    mbar_init(&sm.dotted, kEWarps);
    mbar_init(&sm.mma_done, 1);
    fence_mbar_init();
    sm.fail = 0;
  }
  if (warp == kWarpMma) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.taddr)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t const tmem = sm.taddr;
  // FP16: the A scale per flavour f from the tile copies' maxima, x[1 - f]
  // (rows S) and y[f] (rows Y): |D| <= 12 |Y| |S| <= 24 max|Y| max|S|
  float ascale0 = 1.f, ascale1 = 1.f;
  if constexpr (kF16) {
    const float* tx = tb.x32[pi] + f32_tile_floats(geo.V);
    const float* ty = tb.y32 + f32_tile_floats(geo.V);
    ascale0 = f16_scale(24.f * tx[1] * ty[0]);
    ascale1 = f16_scale(24.f * tx[0] * ty[1]);
  }

  // issue tracking for the teardown after a failure
  int rows_issued_s = -1, rows_issued_y = -1;  // last S block / Y p-block use issued
  int b_issued = -1;
  bool mma_any = false;

  if (warp == kWarpRows) {
    // ---- input rows ---------------------------------------------------------
    // per phase, in the order the D warps use them: the Y rows of p-block bp,
    // then the S rows of its three blocks. A wait here is for the ring slot
    // of a use two (Y) or three (S) steps back, whose readers need only rows
    // issued before it.
    if (lane == 0 && nph > 0) {
      bool ok = true;
      for (int P = 0; ok && P < nph; ++P) {
        int const f = P & 1;
        long long const tile = blockIdx.x + (long long)(P >> 1) * gridDim.x;
        for (int bp = 0; ok && bp < 3; ++bp) {
          for (int h = 0; ok && h < 2; ++h) {
            int const uy = (P * 3 + bp) * 2 + h, ys = uy % kYSlots;
            if (!wait_or_fail(&sm.y_empty[ys], (uint32_t)(((uy / kYSlots) & 1) ^ 1), fail)) { ok = false; break; }
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&sm.y_full[ys], kYRows * kRowBytes);
            for (int r = 0; r < kYRows; ++r)
              bulk_g2s(sm.Y[ys][r], row_ptr(y32, f, 4 * bp + 2 * h + r, tile), kRowBytes, &sm.y_full[ys]);
            rows_issued_y = uy;
          }
          for (int bq = 0; ok && bq < kBlocksQ; ++bq) {
            int const us = P * kBlocks + bp * kBlocksQ + bq, ss = us % kSGroups;
            if (!wait_or_fail(&sm.s_empty[ss], (uint32_t)(((us / kSGroups) & 1) ^ 1), fail)) { ok = false; break; }
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&sm.s_full[ss], kRowsPerGroup * kRowBytes);
            for (int r = 0; r < kRowsPerGroup; ++r)
              bulk_g2s(sm.S[ss][r], row_ptr(x32, 1 - f, 4 * bq + r, tile), kRowBytes, &sm.s_full[ss]);
            rows_issued_s = us;
          }
        }
      }
    }
  } else if (warp == kWarpB) {
    // ---- B chunks -------------------------------------------------------------
    if (lane == 0) {
      int bc = 0;
      bool ok = true;
      for (int P = 0; ok && P < nph; ++P) {
        constexpr int kBP = OpT<kF16>::kBParts;
        const unsigned char* src =
            static_cast<const unsigned char*>(btu) + ((size_t)pi * 2 + (P & 1)) * kChunks * kBP * Sm::kBPartB;
        for (int c = 0; c < kChunks; ++c, ++bc) {
          int const st = bc % kSt;
          if (!wait_or_fail(&sm.a_empty[st], (uint32_t)(((bc / kSt) & 1) ^ 1), fail)) { ok = false; break; }
          fence_proxy_async_smem();
          mbar_arrive_expect_tx(&sm.b_full[st], kBP * Sm::kBPartB);
          bulk_g2s(sm.B[st][0], src + (size_t)c * kBP * Sm::kBPartB, kBP * Sm::kBPartB, &sm.b_full[st]);
          b_issued = bc;
        }
      }
    }
  } else if (warp == kWarpMma) {
    // ---- MMA issue ----------------------------------------------------------------
    // The tensor pipe runs the six MMAs of a chunk in about 500 cycles, so the
    // issuing thread's own per-chunk work has to stay well below that: the
    // stage descriptors differ only in their start address (bits 0-13, in
    // 16-byte units, no carry below 256 KB), so they are formed once and
    // advanced by constants; ring positions and phases are counters.
    if (lane == 0) {
      uint64_t const a_desc0 = sdesc(smem_u32(sm.A[0][0]), (kM / 8) * 128, 128);
      uint64_t const b_desc0 = sdesc(smem_u32(sm.B[0][0]), (kBtN / 8) * 128, 128);
      // in 16-byte units: stage to stage, hi to lo part, and (TF32, two
      // k-steps of 8 per chunk) k-step to k-step: two core columns, 2*16*128
      // and 2*20*128 bytes. FP16: one k-step of 16 per chunk (the chunk's two
      // core columns of 8 k)
      constexpr uint64_t kAStage16 = 2 * Sm::kAPartB / 16, kALo16 = Sm::kAPartB / 16, kAK16 = 2 * (kM / 8) * 128 / 16;
      constexpr uint64_t kBStage16 = OpT<kF16>::kBParts * Sm::kBPartB / 16, kBLo16 = Sm::kBPartB / 16,
                         kBK16 = 2 * (kBtN / 8) * 128 / 16;
      int as = 0, bs = 0;
      uint32_t aph = 0, bph = 0;
      uint32_t const dc = tmem + kCorrCol;
      bool ok = true;
      for (int P = 0; ok && P < nph; ++P) {
        // first half into main buffer P&1 (phase P-1's second half, free once
        // folded), second half into buffer (P+1)&1 (free once dotted)
        if (!wait_or_fail(&sm.folded, (uint32_t)((P & 1) ^ 1), fail)) break;
        tc_fence_after();
        uint32_t const d0 = tmem + (uint32_t)((P & 1) * kBtN), d1 = tmem + (uint32_t)(((P + 1) & 1) * kBtN);
        for (int c = 0; c < kChunks; ++c) {
          if (c == kHalf) {
            if (!wait_or_fail(&sm.dotted, (uint32_t)((P & 1) ^ 1), fail)) { ok = false; break; }
            tc_fence_after();
          }
          if (!wait_or_fail(&sm.a_full[as], aph, fail) || !wait_or_fail(&sm.b_full[bs], bph, fail)) {
            ok = false;
            break;
          }
          tc_fence_after();
          uint32_t const d = c < kHalf ? d0 : d1;
          uint64_t const ahi = a_desc0 + (uint64_t)as * kAStage16, bhi = b_desc0 + (uint64_t)bs * kBStage16;
          // hi.hi into the main buffer, hi.lo and lo.hi into the correction
          // accumulator
          if constexpr (kF16) {
            mma_f16(d, ahi, bhi, (c != 0 && c != kHalf) ? 1u : 0u);
            mma_f16(dc, ahi, bhi + kBLo16, c ? 1u : 0u);
            mma_f16(dc, ahi + kALo16, bhi, 1u);
            mma_f16(dc, ahi, bhi + 2 * kBLo16, 1u);  // hi.lo2
          } else {
            mma_tf32(d, ahi, bhi, (c != 0 && c != kHalf) ? 1u : 0u);
            mma_tf32(dc, ahi, bhi + kBLo16, c ? 1u : 0u);
            mma_tf32(dc, ahi + kALo16, bhi, 1u);
            mma_tf32(d, ahi + kAK16, bhi + kBK16, 1u);
            mma_tf32(dc, ahi + kAK16, bhi + kBK16 + kBLo16, 1u);
            mma_tf32(dc, ahi + kAK16 + kALo16, bhi + kBK16, 1u);
          }
          mma_any = true;
          mma_commit(&sm.a_empty[as]);  // also frees B stage bs (= as)
          if (++as == kSt) { as = 0; aph ^= 1u; }
          if (++bs == kSt) { bs = 0; bph ^= 1u; }
        }
        if (!ok) break;
        mma_commit(&sm.acc_full);
      }
    }
  } else if (warp < kWarpE0) {
    // ---- D formation ----------------------------------------------------------------
    int const grp = (warp - kWarpD0) / kDGroup;  // chunks c = grp, grp + 2, ...
    int const j = (warp - kWarpD0) % kDGroup;    // the chunk's j-th pair of (p, q)
    int const s = lane;
    bool ok = true;
    float y[24];  // this lane's Y row p: loaded at a p-block's first chunk, kept for its three
    for (int P = 0; ok && P < nph; ++P) {
      long long const tile = blockIdx.x + (long long)(P >> 1) * gridDim.x;
      int const nvalid = (int)min((long long)kSites, geo.V - tile * kSites);
      for (int c = grp; c < kChunks; c += kDWarps / kDGroup) {
        // chunk c is half c & 1 (= grp) of block b = (bp, bq): this warp's
        // pair is p = 4 bp + 2 grp + j/2 (row p_in of the Y group) and
        // q = 4 bq + q_in, q_in + 1 (rows of the S group), q_in = 2 (j & 1)
        int const b = c >> 1, bp = b / kBlocksQ, bq = b - bp * kBlocksQ;
        int const uy = (P * 3 + bp) * 2 + grp, ys = uy % kYSlots;  // this group's half
        int const us = P * kBlocks + b, ss = us % kSGroups;
        if (bq == 0) ok = ok && wait_or_fail(&sm.y_full[ys], (uint32_t)((uy / kYSlots) & 1), fail);
        ok = ok && wait_or_fail(&sm.s_full[ss], (uint32_t)((us / kSGroups) & 1), fail);
        int const ac = P * kChunks + c, as = ac % kSt;
        if (!ok || !wait_or_fail(&sm.a_empty[as], (uint32_t)(((ac / kSt) & 1) ^ 1), fail)) { ok = false; break; }
        int const p_in = j >> 1, q_in = 2 * (j & 1);  // rows of the Y half and of the S group
        // k = 4j .. 4j+3 of the chunk, row (mu*32 + s). TF32: core column j,
        // the whole 16-byte row; FP16: core column j/2, its half j&1 (8 bytes)
        unsigned char* Ahi = sm.A[as][0] + (kF16 ? (j >> 1) * 2048 + s * 16 + 8 * (j & 1) : j * 2048 + s * 16);
        unsigned char* Alo = sm.A[as][1] + (kF16 ? (j >> 1) * 2048 + s * 16 + 8 * (j & 1) : j * 2048 + s * 16);
        if (s < nvalid) {
          if (bq == 0) {
            const float* Yr = sm.Y[ys][p_in] + f32_tile_off(s, 0);
            float const sc = kF16 ? ((P & 1) ? ascale1 : ascale0) : 1.f;  // FP16: D scaled through Y
#pragma unroll
            for (int c4 = 0; c4 < 6; ++c4) {
              float4 const a = *reinterpret_cast<const float4*>(Yr + c4 * 64);
              y[4 * c4] = sc * a.x; y[4 * c4 + 1] = sc * a.y; y[4 * c4 + 2] = sc * a.z; y[4 * c4 + 3] = sc * a.w;
            }
          }
          float d[4][4];  // [mu][pq0 re, pq0 im, pq1 re, pq1 im]
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float* Sr = sm.S[ss][q_in + h] + f32_tile_off(s, 0);
            float x[24];
#pragma unroll
            for (int c4 = 0; c4 < 6; ++c4) {
              float4 const bb = *reinterpret_cast<const float4*>(Sr + c4 * 64);
              x[4 * c4] = bb.x; x[4 * c4 + 1] = bb.y; x[4 * c4 + 2] = bb.z; x[4 * c4 + 3] = bb.w;
            }
            // O[s1][s2] = sum_c Y[s1][c] conj(S[s2][c]) for s2 = s1^2 (a) and 3-s1 (b),
            // as packed FP32 pairs: with w = (Re Y, Im Y), U = sum_c w Re S and
            // V = sum_c w Im S (the S part broadcast), Re O = U.x + V.y and
            // Im O = U.y - V.x -- two packed FMAs per (c, s2). D_mu = sum_s1
            // i^((2 - g5g_ph(mu, s1)) & 3) O[s1][s2] (s2 = a for mu = 0, 3; b for
            // mu = 1, 2), i.e. D_0 = a0 + a1 - a2 - a3, D_3 = i (a1 + a3 - a0 - a2),
            // D_1 = -i (b0 + b1 + b2 + b3), D_2 = b0 - b1 + b2 - b3: the b
            // products are summed per parity of s1 inside the FMA chains.
            float a[4][2];
            float2 ube = make_float2(0.f, 0.f), vbe = ube, ubo = ube, vbo = ube;
#pragma unroll
            for (int s1 = 0; s1 < 4; ++s1) {
              float2 ua = make_float2(0.f, 0.f), va = ua;
#pragma unroll
              for (int cc = 0; cc < 3; ++cc) {
                float2 const w = make_float2(y[2 * (3 * s1 + cc)], y[2 * (3 * s1 + cc) + 1]);
                int const sa = 2 * (3 * (s1 ^ 2) + cc), sb = 2 * (3 * (3 - s1) + cc);
                ua = __ffma2_rn(w, make_float2(x[sa], x[sa]), ua);
                va = __ffma2_rn(w, make_float2(x[sa + 1], x[sa + 1]), va);
                if (s1 & 1) {
                  ubo = __ffma2_rn(w, make_float2(x[sb], x[sb]), ubo);
                  vbo = __ffma2_rn(w, make_float2(x[sb + 1], x[sb + 1]), vbo);
                } else {
                  ube = __ffma2_rn(w, make_float2(x[sb], x[sb]), ube);
                  vbe = __ffma2_rn(w, make_float2(x[sb + 1], x[sb + 1]), vbe);
                }
              }
              a[s1][0] = ua.x + va.y; a[s1][1] = ua.y - va.x;
            }
            float const ber = ube.x + vbe.y, bei = ube.y - vbe.x;
            float const bor = ubo.x + vbo.y, boi = ubo.y - vbo.x;
            float const a01r = a[0][0] + a[1][0], a01i = a[0][1] + a[1][1];
            float const a23r = a[2][0] + a[3][0], a23i = a[2][1] + a[3][1];
            float const a13r = a[1][0] + a[3][0], a13i = a[1][1] + a[3][1];
            float const a02r = a[0][0] + a[2][0], a02i = a[0][1] + a[2][1];
            d[0][2 * h] = a01r - a23r; d[0][2 * h + 1] = a01i - a23i;
            d[3][2 * h] = a02i - a13i; d[3][2 * h + 1] = a13r - a02r;  // i (a13 - a02)
            d[1][2 * h] = bei + boi;   d[1][2 * h + 1] = -(ber + bor);  // -i (be + bo)
            d[2][2 * h] = ber - bor;   d[2][2 * h + 1] = bei - boi;
          }
#pragma unroll
          for (int mu = 0; mu < 4; ++mu) {
            if constexpr (kF16) {
              uint2 hi, lo;
              f16_split2(d[mu][0], d[mu][1], hi.x, lo.x);
              f16_split2(d[mu][2], d[mu][3], hi.y, lo.y);
              *reinterpret_cast<uint2*>(Ahi + mu * 32 * 16) = hi;
              *reinterpret_cast<uint2*>(Alo + mu * 32 * 16) = lo;
            } else {
              float4 hi, lo;
              hi.x = tf32_round(d[mu][0]); hi.y = tf32_round(d[mu][1]);
              hi.z = tf32_round(d[mu][2]); hi.w = tf32_round(d[mu][3]);
              lo.x = tf32_round(d[mu][0] - hi.x); lo.y = tf32_round(d[mu][1] - hi.y);
              lo.z = tf32_round(d[mu][2] - hi.z); lo.w = tf32_round(d[mu][3] - hi.w);
              *reinterpret_cast<float4*>(Ahi + mu * 32 * 16) = hi;
              *reinterpret_cast<float4*>(Alo + mu * 32 * 16) = lo;
            }
          }
        } else {
#pragma unroll
          for (int mu = 0; mu < 4; ++mu) {
            if constexpr (kF16) {
              *reinterpret_cast<uint2*>(Ahi + mu * 32 * 16) = make_uint2(0u, 0u);
              *reinterpret_cast<uint2*>(Alo + mu * 32 * 16) = make_uint2(0u, 0u);
            } else {
              *reinterpret_cast<float4*>(Ahi + mu * 32 * 16) = make_float4(0.f, 0.f, 0.f, 0.f);
              *reinterpret_cast<float4*>(Alo + mu * 32 * 16) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
          }
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&sm.a_full[as]);
          // every D warp reads each S block in one chunk; a group reads its
          // Y half in three (bq = 0..2)
          mbar_arrive(&sm.s_empty[ss]);
          if (bq == kBlocksQ - 1) mbar_arrive(&sm.y_empty[ys]);
        }
      }
    }
  } else {
    // ---- epilogue -----------------------------------------------------------------------
    int const quad = warp & 3;  // the TMEM lanes this warp may access; mu = quad
    int const s = lane;
    uint32_t const lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
    const int gsx[4] = {tb.gsx[pi][0], tb.gsx[pi][1], tb.gsx[pi][2], tb.gsx[pi][3]};
    const int yv[4] = {tb.yv[pi][0], tb.yv[pi][1], tb.yv[pi][2], tb.yv[pi][3]};
    const double* __restrict__ wq = kGeneric ? nullptr : args.w + (size_t)pi * geo.V * 3 * HLBL_QED_NW;
    const float* __restrict__ cg =
        kGeneric ? static_cast<const float*>(args.coef) + (size_t)pi * args.coef_stride : nullptr;
    double const xu = args.xunit;
    SiteQ q;
#pragma unroll
    for (int r = 0; r < 4; ++r) q.ym[r] = (float)(coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]) * xu);
    Neu run0, run1;
    for (int P = 0; P < nph; ++P) {
      long long const tile = blockIdx.x + (long long)(P >> 1) * gridDim.x;
      long long const v = tile * kSites + s;
      bool const valid = v < geo.V;
      if (!kGeneric && (P & 1) == 0) {
        // the row's site data, for both flavours of the tile
        long long const vv = valid ? v : geo.V - 1;
        int rel[4];
        rel_coords(geo, gsx, vv, rel);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          q.xm[r] = (float)(coord_map(rel[r], geo.global[r]) * xu);
          q.xmy[r] = (float)(coord_map_diff(rel[r], yv[r], geo.global[r]) * xu);
          q.zh[r] = (float)coord_map_zerohalf(rel[r], geo.global[r]);
        }
#pragma unroll
        for (int e = 0; e < 3; ++e)
#pragma unroll
          for (int k = 0; k < HLBL_QED_NW; ++k) q.w[e][k] = (float)wq[((size_t)vv * 3 + e) * HLBL_QED_NW + k];
      }
      if (!wait_or_fail(&sm.acc_full, (uint32_t)(P & 1), fail)) break;
      tc_fence_after();
      uint32_t const c0 = (uint32_t)((P & 1) * kBtN), c1 = (uint32_t)(((P + 1) & 1) * kBtN);
      // fold the second half and the corrections into the first half
#pragma unroll 1
      for (int jj = 0; jj < 10; ++jj) {
        float m[16], h[16], k[16];
        tmem_ld16(lane_addr + c0 + 16 * jj, m);
        tmem_ld16(lane_addr + c1 + 16 * jj, h);
        tmem_ld16(lane_addr + kCorrCol + 16 * jj, k);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) m[i] = (m[i] + h[i]) + k[i];
        tmem_st16(lane_addr + c0 + 16 * jj, m);
      }
      tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.folded);
      tc_fence_after();
      float a;
      if constexpr (kGeneric) {
        // the row (mu = quad, site s of the tile); pad sites' coefficients are zero
        a = epilogue_row_generic(lane_addr, c0, cg + coef32_index(tile * kSites, quad, 0) + (size_t)s * 4);
      } else {
        switch (quad) {
          case 0: a = epilogue_row<0>(lane_addr, c0, q); break;
          case 1: a = epilogue_row<1>(lane_addr, c0, q); break;
          case 2: a = epilogue_row<2>(lane_addr, c0, q); break;
          default: a = epilogue_row<3>(lane_addr, c0, q); break;
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.dotted);
      if constexpr (kF16) a *= 1.f / (((P & 1) ? ascale1 : ascale0) * bscale[2 * pi + (P & 1)]);  // powers of two: exact
      if (valid) {
        if (P & 1) run1.add(-(double)a);
        else run0.add(-(double)a);
      }
    }
    if (!*fail) {
      // fixed-order compensated reduction over the epilogue's 128 threads
      Neu r0 = run0, r1 = run1;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double const s0v = __shfl_down_sync(0xffffffffu, r0.s, o), c0v = __shfl_down_sync(0xffffffffu, r0.c, o);
        double const s1v = __shfl_down_sync(0xffffffffu, r1.s, o), c1v = __shfl_down_sync(0xffffffffu, r1.c, o);
        r0.add(s0v); r0.c += c0v;
        r1.add(s1v); r1.c += c1v;
      }
      if (lane == 0) {
        int const ew = warp - kWarpE0;
        sm.red[ew][0][0] = r0.s; sm.red[ew][0][1] = r0.c;
        sm.red[ew][1][0] = r1.s; sm.red[ew][1][1] = r1.c;
      }
    }
  }

  // ---- teardown ----------------------------------------------------------------------------
  tc_fence_before();
  __syncthreads();
  if (*fail) {
    // let nothing this CTA started outlive it (each wait bounded)
    if (warp == kWarpRows && lane == 0) {
      for (int u = rows_issued_s - kSGroups + 1; u <= rows_issued_s; ++u)
        if (u >= 0) mbar_wait(&sm.s_full[u % kSGroups], (uint32_t)((u / kSGroups) & 1));
      for (int u = rows_issued_y - kYSlots + 1; u <= rows_issued_y; ++u)
        if (u >= 0) mbar_wait(&sm.y_full[u % kYSlots], (uint32_t)((u / kYSlots) & 1));
    }
    if (warp == kWarpB && lane == 0)
      for (int u = b_issued - kSt + 1; u <= b_issued; ++u)
        if (u >= 0) mbar_wait(&sm.b_full[u % kSt], (uint32_t)((u / kSt) & 1));
    if (warp == kWarpMma && lane == 0 && mma_any) {
      mma_commit(&sm.mma_done);
      mbar_wait(&sm.mma_done, 0);
    }
    if (t == 0 && err) atomicExch(err, kErrWaitTimeout);
  } else if (t == kWarpE0 * 32) {
    for (int f = 0; f < 2; ++f) {
      Neu acc;
      for (int w = 0; w < kEWarps; ++w) { acc.add(sm.red[w][f][0]); acc.c += sm.red[w][f][1]; }
      partials[((size_t)pi * gridDim.x + blockIdx.x) * 2 + f] = acc.get();
    }
  }
  __syncthreads();
  tc_fence_after();
  if (warp == kWarpMma)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// B operand of the tensor-core pass 2, from the gamma-inserted pass-1 sums:
// per (pair, flavour) and chunk of 16 k, the 160 x 16 block of Bt^T as TF32
// hi and lo parts in the K-major core-matrix layout (core (kg, n/8) at
// (kg*20 + n/8)*128 bytes, row n%8 at 16 bytes, k%4 at 4 bytes). The values
// are bt_build_kernel's.
__global__ void btu_build_kernel(const double* __restrict__ g, int nf, float* __restrict__ btu) {
  int const fl = blockIdx.y, pi = blockIdx.z;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kBtK * kBtN || fl >= nf) return;
  const double* g_dzu = g + ((size_t)pi * nf + fl) * kGLen;
  const double* g_dzsu = g_dzu + kGDzuLen;
  int const k = i / kBtN, n = i % kBtN;
  // k within chunk c: 4 jj + 2 hh + e for the pair (p, q) the D formation
  // puts there (block b = c/2 of 4 p x 4 q, half c & 1)
  int const cc = k / kKc, kl = k % kKc, jj = kl >> 2, hh = (kl >> 1) & 1, e = kl & 1;
  int const bb = cc >> 1, bbp = bb / kBlocksQ, bbq = bb - bbp * kBlocksQ;
  int const p = 4 * bbp + 2 * (cc & 1) + (jj >> 1), q = 4 * bbq + 2 * (jj & 1) + hh;
  int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
  int const sq = q / 3, cq = q % 3;
  int sq2 = 0;
#pragma unroll
  for (int s = 0; s < 4; ++s)
    if (gg5_src(lam, s) == sq) sq2 = s;
  int const ph = gg5_ph(lam, sq2);
  const double* v = j < 6 ? g_dzu + ((((j * 4 + nu) * 12) + (3 * sq2 + cq)) * 12 + p) * 2
                          : g_dzsu + (((((j - 6) * 4 + nu) * 12) + (3 * sq2 + cq)) * 12 + p) * 2;
  double re, im;
  mul_iph(ph, v[0], v[1], re, im);
  double const x = e == 0 ? re : -im;
  float const hi = __uint_as_float(tf32_rna((float)x));
  float const lo = __uint_as_float(tf32_rna((float)(x - (double)hi)));
  int const c = k / kKc, kk = k % kKc;
  size_t const base = (((size_t)pi * 2 + fl) * kChunks + c) * 2 * kBPart;
  int const off = ((kk >> 2) * (kBtN / 8) + (n >> 3)) * 32 + (n & 7) * 4 + (kk & 3);
  btu[base + off] = hi;
  btu[base + kBPart + off] = lo;
}

// FP16 operands: the B scale per (pair, flavour), 2^(15 - e) with 2^e above
// max |g| (every Bt entry is a component of g times a power of i)
__global__ void bscale_kernel(const double* __restrict__ g, int nf, float* __restrict__ bscale) {
  __shared__ float red[8];
  int const fl = blockIdx.x, pi = blockIdx.y;
  const double* gp = g + ((size_t)pi * nf + fl) * kGLen;
  float m = 0.f;
  for (int i = threadIdx.x; i < kGLen; i += blockDim.x) m = fmaxf(m, fabsf((float)gp[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
    bscale[pi * 2 + fl] = f16_scale(m);
  }
}

// btu_build_kernel's values scaled by bscale, as FP16 hi, lo and lo2 parts
// (each the rounding of the rest of the FP64 value) in the K-major
// core-matrix layout of 8 k (core (k/8, n/8) at (k/8*20 + n/8)*128
// bytes, row n%8 at 16 bytes, k%8 at 2 bytes)
__global__ void btu16_build_kernel(const double* __restrict__ g, int nf, const float* __restrict__ bscale,
                                   __half* __restrict__ btu) {
  int const fl = blockIdx.y, pi = blockIdx.z;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kBtK * kBtN || fl >= nf) return;
  const double* g_dzu = g + ((size_t)pi * nf + fl) * kGLen;
  const double* g_dzsu = g_dzu + kGDzuLen;
  int const k = i / kBtN, n = i % kBtN;
  int const cc = k / kKc, kl = k % kKc, jj = kl >> 2, hh = (kl >> 1) & 1, e = kl & 1;
  int const bb = cc >> 1, bbp = bb / kBlocksQ, bbq = bb - bbp * kBlocksQ;
  int const p = 4 * bbp + 2 * (cc & 1) + (jj >> 1), q = 4 * bbq + 2 * (jj & 1) + hh;
  int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
  int const sq = q / 3, cq = q % 3;
  int sq2 = 0;
#pragma unroll
  for (int s = 0; s < 4; ++s)
    if (gg5_src(lam, s) == sq) sq2 = s;
  int const ph = gg5_ph(lam, sq2);
  const double* v = j < 6 ? g_dzu + ((((j * 4 + nu) * 12) + (3 * sq2 + cq)) * 12 + p) * 2
                          : g_dzsu + (((((j - 6) * 4 + nu) * 12) + (3 * sq2 + cq)) * 12 + p) * 2;
  double re, im;
  mul_iph(ph, v[0], v[1], re, im);
  double const x = (e == 0 ? re : -im) * (double)bscale[pi * 2 + fl];  // a power of two: exact
  __half const hi = __double2half(x);
  double const r1 = x - (double)__half2float(hi);
  __half const lo = __double2half(r1);
  __half const lo2 = __double2half(r1 - (double)__half2float(lo));
  int const off = ((kl >> 3) * (kBtN / 8) + (n >> 3)) * 64 + (n & 7) * 8 + (kl & 7);
  size_t const base = (((size_t)pi * 2 + fl) * kChunks + cc) * 3 * kBPart;
  btu[base + off] = hi;
  btu[base + kBPart + off] = lo;
  btu[base + 2 * kBPart + off] = lo2;
}

}  // namespace tc

size_t tc_smem_bytes() { return sizeof(tc::Smem); }
int tc_threads() { return tc::kThreads; }
size_t tc_btu_floats_per_pair() { return (size_t)2 * tc::kChunks * 2 * tc::kBPart; }

template <bool G, bool F>
static int tc_init_one(int& nb) {
  size_t const smem = sizeof(tc::SmemT<F>);
  cudaError_t e = cudaFuncSetAttribute(tc::p2tc_kernel<G, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "p2tc smem attribute");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, tc::p2tc_kernel<G, F>, tc::kThreads, smem);
  if (e != cudaSuccess) return cuda_fail(e, "p2tc occupancy");
  if (nb < 1) return fail(HLBL_ECUDA, "p2tc kernel cannot be resident (smem %zu)", smem);
  return HLBL_OK;
}

int tc_init(int nsm, int& grid) {
  int nb = 0;
  if (int rc = tc_init_one<false, false>(nb)) return rc;
  if (int rc = tc_init_one<true, false>(nb)) return rc;
  if (int rc = tc_init_one<false, true>(nb)) return rc;
  if (int rc = tc_init_one<true, true>(nb)) return rc;
  // one CTA per SM: each allocates all 512 TMEM columns
  grid = nsm;
  return HLBL_OK;
}

void tc_launch_btu(const double* d_g, int npairs, void* d_btu, bool f16, float* d_bscale, cudaStream_t st) {
  dim3 const gb((kBtK * kBtN + 255) / 256, 2, npairs);
  if (f16) {
    tc::bscale_kernel<<<dim3(2, npairs), 256, 0, st>>>(d_g, 2, d_bscale);
    tc::btu16_build_kernel<<<gb, 256, 0, st>>>(d_g, 2, d_bscale, static_cast<__half*>(d_btu));
  } else {
    tc::btu_build_kernel<<<gb, 256, 0, st>>>(d_g, 2, static_cast<float*>(d_btu));
  }
}

void tc_launch_p2(int grid, int npairs, cudaStream_t st, const TcBatch& tb, const Geometry& geo,
                  const P2Args& a, const void* d_btu, bool f16, const float* d_bscale, double* partials, int* err) {
  dim3 const gr(grid, npairs);
  if (f16) {
    size_t const smem = sizeof(tc::SmemT<true>);
    if (a.coef) tc::p2tc_kernel<true, true><<<gr, tc::kThreads, smem, st>>>(tb, geo, a, d_btu, d_bscale, partials, err);
    else tc::p2tc_kernel<false, true><<<gr, tc::kThreads, smem, st>>>(tb, geo, a, d_btu, d_bscale, partials, err);
  } else {
    size_t const smem = sizeof(tc::SmemT<false>);
    if (a.coef) tc::p2tc_kernel<true, false><<<gr, tc::kThreads, smem, st>>>(tb, geo, a, d_btu, d_bscale, partials, err);
    else tc::p2tc_kernel<false, false><<<gr, tc::kThreads, smem, st>>>(tb, geo, a, d_btu, d_bscale, partials, err);
  }
}

long long tc_tiles(long long V) { return (V + tc::kSites - 1) / tc::kSites; }

}  // namespace hg
