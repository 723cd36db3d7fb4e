// capi.cu -- the C ABI of libhlbl_gb300.so: the contraction context, its
// work buffers and stream, kernel launch plumbing, and the entry points
// declared in include/hlbl_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "contract_kernels.cuh"
#include "hlbl_gb300.h"
#include "hlbl_gb300_rng.h"
#include "hlbl_internal.h"
#include "p2_tc.h"
#include "pieces_2p2.h"
#include "qed_provider.cuh"

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace hg {
namespace sur {
// surrogate.cu: pass 2's weights from the learned surrogate
int launch_surrogate_weights(const hlbl_surrogate* s, const Geometry& geo, const WArgs& wa,
                             double r0, const QedF32& qf, double r64, double* d_w,
                             unsigned long long* d_fallback, cudaStream_t st, int nsm);
double surrogate_r0(const hlbl_surrogate* s);
}  // namespace sur
}  // namespace hg

namespace hg {

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(HLBL_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ---- fixture kernels -------------------------------------------------------
__global__ void fill_uniform_kernel(double* __restrict__ out, Geometry geo, uint64_t seed) {
  long long const n = geo.V * 2 * 12 * 24;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    int const c = (int)(i % 24);
    long long const site = (i / 24) % geo.V;
    int const row = (int)(i / (24 * geo.V));  // f*12 + ia
    long long s = site;
    int lc[4];
    lc[3] = (int)(s % geo.local[3]); s /= geo.local[3];
    lc[2] = (int)(s % geo.local[2]); s /= geo.local[2];
    lc[1] = (int)(s % geo.local[1]); s /= geo.local[1];
    lc[0] = (int)s;
    uint64_t const g = hlbl_rng_site_key(geo.pc[0] * geo.local[0] + lc[0], geo.pc[1] * geo.local[1] + lc[1],
                                         geo.pc[2] * geo.local[2] + lc[2], geo.pc[3] * geo.local[3] + lc[3]);
    out[i] = hlbl_rng_uniform_entry(seed, g, row / 12, row % 12, c);
  }
}

__global__ void fill_gaussian_kernel(double* __restrict__ out, Geometry geo, uint64_t seed) {
  long long const n = geo.V * 2 * 12 * 12;  // complex entries
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    int const c = (int)(i % 12);
    long long const site = (i / 12) % geo.V;
    int const row = (int)(i / (12 * geo.V));
    long long s = site;
    int lc[4];
    lc[3] = (int)(s % geo.local[3]); s /= geo.local[3];
    lc[2] = (int)(s % geo.local[2]); s /= geo.local[2];
    lc[1] = (int)(s % geo.local[1]); s /= geo.local[1];
    lc[0] = (int)s;
    uint64_t const g = hlbl_rng_site_key(geo.pc[0] * geo.local[0] + lc[0], geo.pc[1] * geo.local[1] + lc[1],
                                         geo.pc[2] * geo.local[2] + lc[2], geo.pc[3] * geo.local[3] + lc[3]);
    double re, im;
    hlbl_rng_gaussian_entry(seed, g, row / 12, row % 12, c, &re, &im);
    reinterpret_cast<double2*>(out)[i] = make_double2(re, im);
  }
}

// Diagnostic for the bounded waits: an mbarrier told to expect 16 bytes that
// never come, so the phase never completes; the wait gives up, sets the
// error flag and the kernel returns (nothing is in flight).
__global__ void wait_timeout_selftest_kernel(int* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(&bar, 16);
  }
  __syncthreads();
  bool const ok = mbar_wait(&bar, 0);
  if (!ok && threadIdx.x == 0) atomicExch(err, kErrWaitTimeout);
}

// The FP32 tile copy of one block ([f][ia][tile][2][6][16][4] floats), with the
// conversion pass 1 uses; sites past V in the last tile are left untouched.
// FP64 block -> FP32 tile copy. A warp takes one (row, 32-site tile, 16-byte
// group c4): lane = site of the tile, so each lane reads one 32-byte sector
// of the block and the warp writes two contiguous 256-byte runs of the copy;
// 32-bit index arithmetic (V * 6 < 2^31), blockIdx.y = row (f, ia).
__global__ void f32_tile_copy_kernel(const double* __restrict__ blk, Geometry geo, float* __restrict__ out) {
  unsigned const nt32 = (unsigned)((geo.V + 31) / 32), V = (unsigned)geo.V;
  unsigned const n = nt32 * 6 * 32;  // (tile, c4, lane)
  int const row = blockIdx.y;
  const double* __restrict__ src_row = blk + (size_t)row * geo.V * 24;
  float* __restrict__ dst_row = out + (size_t)row * nt32 * (32 * 24);
  float m = 0.f;  // the largest magnitude this thread converts
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned const lane = i & 31, k = i >> 5, c4 = k % 6, t32 = k / 6;
    unsigned const site = t32 * 32 + lane;
    if (site >= V) continue;  // the copy's padding past the last site is never read
    const double2* src = reinterpret_cast<const double2*>(src_row + (size_t)site * 24 + 4 * c4);
    double2 const v0 = src[0], v1 = src[1];
    float4 const f = make_float4(f64_to_f32(v0.x), f64_to_f32(v0.y), f64_to_f32(v1.x), f64_to_f32(v1.y));
    *reinterpret_cast<float4*>(dst_row + (size_t)t32 * (32 * 24) + f32_tile_off((int)lane, (int)c4)) = f;
    m = fmaxf(m, fmaxf(fmaxf(fabsf(f.x), fabsf(f.y)), fmaxf(fabsf(f.z), fabsf(f.w))));
  }
  // the flavour's largest magnitude into the copy's trailer (zeroed before
  // the launch; non-negative floats order as their bit patterns)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f)
    atomicMax(reinterpret_cast<int*>(out + f32_tile_floats(geo.V)) + row / 12, __float_as_int(m));
}

// ---- launch plumbing -------------------------------------------------------
template <typename T, int NF, int TS>
struct P1Launch {
  static constexpr int threads = NF * 144;
  static constexpr size_t smem = p1_smem_bytes<T, NF, TS>();
  static int init(int nsm, int& grid) {
    cudaError_t e = cudaFuncSetAttribute(p1_kernel<T, NF, TS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // all of the unified L1/shared storage as shared memory: two FP32 CTAs per SM
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(p1_kernel<T, NF, TS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_fail(e, "p1 smem attribute");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, p1_kernel<T, NF, TS>, threads, smem);
    if (e != cudaSuccess) return cuda_fail(e, "p1 occupancy");
    if (nb < 1) return fail(HLBL_ECUDA, "p1 kernel cannot be resident (smem %zu)", smem);
    grid = nb * nsm;
    return HLBL_OK;
  }
  static void launch(int grid, cudaStream_t st, const double* y, const PairBatch& b,
                     const Geometry& geo, int f0, double* partials, int* err, float* y32 = nullptr) {
    p1_kernel<T, NF, TS><<<dim3(grid, b.n), threads, smem, st>>>(y, b, geo, f0, partials, err, y32);
  }
  static long long tiles(long long V) { return (V + TS - 1) / TS; }
};

template <typename T, int NF, int TS>
struct P2Launch {
  static constexpr int threads = NF * 160;
  static constexpr size_t smem = p2_smem_bytes<T, NF, TS>();
  static int init(int nsm, int& grid) {
    cudaError_t e = cudaFuncSetAttribute(p2_kernel<T, NF, TS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "p2 smem attribute");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, p2_kernel<T, NF, TS>, threads, smem);
    if (e != cudaSuccess) return cuda_fail(e, "p2 occupancy");
    if (nb < 1) return fail(HLBL_ECUDA, "p2 kernel cannot be resident (smem %zu)", smem);
    grid = nb * nsm;
    return HLBL_OK;
  }
  static void launch(int grid, cudaStream_t st, const double* y, const PairBatch& b,
                     const Geometry& geo, const P2Args& a, const T* bt, double* partials, int* err) {
    p2_kernel<T, NF, TS><<<dim3(grid, b.n), threads, smem, st>>>(y, b, geo, a, bt, partials, err);
  }
  static long long tiles(long long V) { return (V + TS - 1) / TS; }
};

// tile sizes per precision (the FP32 two-flavour kernels have a second tile
// size each, which the autotuner may choose)
using P1D2 = P1Launch<double, 2, 8>;
using P1D1 = P1Launch<double, 1, 8>;
using P1F2 = P1Launch<float, 2, 8>;
using P1F2s = P1Launch<float, 2, 4>;
using P1F1 = P1Launch<float, 1, 8>;
using P2D2 = P2Launch<double, 2, 4>;
using P2D1 = P2Launch<double, 1, 4>;
using P2F2 = P2Launch<float, 2, 4>;
using P2F2s = P2Launch<float, 2, 2>;
using P2F1 = P2Launch<float, 1, 4>;

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int make_geometry(const int global[4], const int local[4], const int pc[4], Geometry& g) {
  long long V = 1;
  for (int r = 0; r < 4; ++r) {
    if (local[r] < 1 || global[r] < 1 || pc[r] < 0)
      return fail(HLBL_EINVAL, "geometry: extents must be positive, coordinates >= 0");
    if ((long long)(pc[r] + 1) * local[r] > global[r])
      return fail(HLBL_EINVAL, "geometry: rank %d of local extent %d exceeds global %d in dir %d",
                  pc[r], local[r], global[r], r);
    g.local[r] = local[r];
    g.global[r] = global[r];
    g.pc[r] = pc[r];
    V *= local[r];
  }
  g.V = V;
  return HLBL_OK;
}

}  // namespace hg

using namespace hg;

struct hlbl_ctx {
  int device = 0;
  int nsm = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  Geometry geo{};
  hlbl_qed_params qp{};
  int grid_p1d2 = 0, grid_p1d1 = 0, grid_p1f2 = 0, grid_p1f1 = 0, grid_p1f2s = 0;
  int grid_p2d2 = 0, grid_p2d1 = 0, grid_p2f2 = 0, grid_p2f1 = 0, grid_p2f2s = 0;
  int p1_small = 0, p2_small = 0;  // FP32 tile variants chosen (autotuner)
  // FP32 two-flavour pass 2 on the tensor cores (p2_tc.cu); off: CUDA cores
  int tc = 1;
  int grid_tc = 0;
  int grid_p1f[kP1f32Variants] = {};  // pass 1 on FP32 tile copies, per variant (p2_tc.h)
  int p1f_var = 1;
  int group_f32 = 0;          // pairs per launch on the FP32-copy path (0: kMaxBatch)
  float* d_x32 = nullptr;     // FP32 tile copies: [1 + pair][f32 block] (y first)
  size_t x32_floats = 0;
  float* d_btu = nullptr;     // tensor-core B operand [kMaxBatch][tc_btu_floats_per_pair]
  float* d_bscale = nullptr;  // FP16 operands: B scale [kMaxBatch][2]
  int tc16 = 1;               // FP16 operands in the FP32-copy path's pass 2 (hlbl_ctx_set_tc_fp16)
  // staging of host blocks on a side stream (hlbl_stage_async)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t stage_ev = nullptr;
  cudaEvent_t compute_ev = nullptr;
  bool stage_pending = false;
  bool capturing = false;
  int max_grid = 0;
  double* d_part1 = nullptr;  // [max_grid][2][2880]
  double* d_part2 = nullptr;  // [max_grid][2]
  double* d_dz = nullptr;     // [2][2880]
  double* d_g = nullptr;      // [2][11520]
  void* d_bt = nullptr;       // [2][288*160] of double (float uses half of it)
  double* d_w = nullptr;      // QED weights [V][3][6]
  long long w_cap = 0;        // sites d_w holds
  // the QED kernel (hlbl_ctx_set_qed_kernel): the stand-in's closed form, or
  // a provider through the generic coefficient path
  int qed_kind = kQedStandInClosed;
  double* d_dense64 = nullptr;  // the dense test weight's table [13][384]
  float* d_dense32 = nullptr;
  void* d_coef = nullptr;       // generic path: coefficients of a pair group
#ifdef HLBL_WITH_KQED
  QED_kernel_temps kq{};        // a linked KQED's temps (initialise())
  bool kq_ready = false;
#endif
  size_t coef_cap = 0;          // bytes of d_coef
  int batch_group = 0;        // pairs per batched launch (0: kMaxBatch)
  int qed_mode = HLBL_QED_EXACT;
  // FP32 path, exact weight: FP32 quadrature outside qed_r64 (FP64 inside)
  int qed_fp32 = 1;
  double qed_r64 = 0.1;
  QedF32 qf{};                // the weight's FP32 quadrature tables (from qp)
  const hlbl_surrogate* sur = nullptr;
  double sur_r0 = 0.0;
  unsigned long long* d_fallback = nullptr;  // rows evaluated exactly inside r0
  double* d_out = nullptr;    // [2]
  double* h_out = nullptr;    // pinned [2]
  int* d_err = nullptr;       // kernels' error flag (a bounded wait gave up)
  // 2+2 pieces: work buffers, and the device results of the blocking calls
  hg::P22* p22 = nullptr;
  double p22_r64 = 0.0;       // FP32 2+2 path: FP64 QED weight within this radius
  double* d_p22_out = nullptr;
  size_t p22_out_cap = 0;     // doubles
  // optional per-kernel timing with CUDA events on the launching stream
  bool profiling = false;
  cudaEvent_t ev[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [pass][begin/end]
  double prof_ms[2] = {0, 0};
  long long prof_n[2] = {0, 0};
  int prof_pending[2] = {0, 0};
};

namespace hg {

// Profiling: events around one kernel; the elapsed time is collected at
// the next prof_begin of that pass (or by hlbl_ctx_kernel_times).
void prof_collect(hlbl_ctx* c, int pass) {
  if (!c->profiling || c->prof_pending[pass] == 0) return;
  float ms = 0.f;
  if (cudaEventSynchronize(c->ev[pass][1]) == cudaSuccess &&
      cudaEventElapsedTime(&ms, c->ev[pass][0], c->ev[pass][1]) == cudaSuccess) {
    c->prof_ms[pass] += ms;
    c->prof_n[pass] += 1;
  }
  c->prof_pending[pass] = 0;
}
void prof_begin(hlbl_ctx* c, int pass) {
  if (!c->profiling || c->capturing) return;
  prof_collect(c, pass);
  cudaEventRecord(c->ev[pass][0], c->stream);
}
void prof_end(hlbl_ctx* c, int pass) {
  if (!c->profiling || c->capturing) return;
  cudaEventRecord(c->ev[pass][1], c->stream);
  c->prof_pending[pass] = 1;
}

// Thread blocks per pair: the resident grid shared among the batch's pairs,
// at most one tile each.
int per_pair_grid(int resident, int npairs, long long tiles) {
  long long g = std::max(1, resident / std::max(1, npairs));
  return (int)std::min(g, tiles);
}

bool use_tc(const hlbl_ctx* c, int precision, int nf) { return precision == HLBL_FP32 && nf == 2 && c->tc; }

// FP32 tile copies for y and `npairs` partners (grown outside graph capture).
int ensure_x32(hlbl_ctx* c, const Geometry& geo, int npairs) {
  size_t const need = (size_t)(1 + npairs) * f32_block_floats(geo.V);
  if (need <= c->x32_floats) return HLBL_OK;
  if (c->capturing) return fail(HLBL_ESTATE, "FP32 tile buffer too small during graph capture");
  cudaStreamSynchronize(c->stream);
  cudaFree(c->d_x32);
  c->d_x32 = nullptr;
  c->x32_floats = 0;
  cudaError_t e = cudaMalloc(&c->d_x32, sizeof(float) * need);
  if (e != cudaSuccess) return fail(HLBL_ENOMEM, "FP32 tile buffer (%zu bytes): %s", sizeof(float) * need, cudaGetErrorString(e));
  c->x32_floats = need;
  return HLBL_OK;
}
float* x32_block(hlbl_ctx* c, const Geometry& geo, int slot) { return c->d_x32 + (size_t)slot * f32_block_floats(geo.V); }

// Pass 1 + reduction + gamma insertion + Bt for the batch's pairs, flavours
// [f0, f0+nf). Pair i, flavour fl: dz at d_dz + (i*nf + fl)*kDzLen, g at
// d_g + (i*nf + fl)*kGLen, Bt at d_bt + (i*nf + fl)*kBtK*kBtN.
int run_pass1(hlbl_ctx* c, const Geometry& geo, const double* y, const PairBatch& b, int f0,
              int nf, int precision, double* add_dzu, double* add_dzsu, bool build_bt) {
  if (c->stage_pending) {  // blocks staged on the side stream must have landed
    cudaError_t e = cudaStreamWaitEvent(c->stream, c->stage_ev, 0);
    if (e != cudaSuccess) return cuda_fail(e, "wait for staged block");
    c->stage_pending = false;
  }
  int grid;
  bool const tcp = use_tc(c, precision, nf) && build_bt;
  PairBatch bb = b;
  float* y32 = nullptr;
  if (tcp) {
    if (int rc = ensure_x32(c, geo, b.n)) return rc;
    y32 = x32_block(c, geo, 0);
    for (int i = 0; i < b.n; ++i) bb.p[i].src32 = x32_block(c, geo, 1 + i);
  }
  prof_begin(c, 0);
  if (precision == HLBL_FP64) {
    if (nf == 2) { grid = per_pair_grid(c->grid_p1d2, b.n, P1D2::tiles(geo.V)); P1D2::launch(grid, c->stream, y, b, geo, f0, c->d_part1, c->d_err); }
    else { grid = per_pair_grid(c->grid_p1d1, b.n, P1D1::tiles(geo.V)); P1D1::launch(grid, c->stream, y, b, geo, f0, c->d_part1, c->d_err); }
  } else {
    if (nf == 2 && c->p1_small) { grid = per_pair_grid(c->grid_p1f2s, b.n, P1F2s::tiles(geo.V)); P1F2s::launch(grid, c->stream, y, bb, geo, f0, c->d_part1, c->d_err, y32); }
    else if (nf == 2) { grid = per_pair_grid(c->grid_p1f2, b.n, P1F2::tiles(geo.V)); P1F2::launch(grid, c->stream, y, bb, geo, f0, c->d_part1, c->d_err, y32); }
    else { grid = per_pair_grid(c->grid_p1f1, b.n, P1F1::tiles(geo.V)); P1F1::launch(grid, c->stream, y, b, geo, f0, c->d_part1, c->d_err); }
  }
  prof_end(c, 0);
  p1_reduce_kernel<<<dim3((kDzLen + kRedOut - 1) / kRedOut, nf, b.n), kRedOut * kRedGrp, 0, c->stream>>>(
      c->d_part1, grid, nf, c->d_dz, add_dzu, add_dzsu);
  if (!build_bt) return HLBL_OK;
  g_build_kernel<<<dim3((kGLen / 2 + 255) / 256, nf, b.n), 256, 0, c->stream>>>(c->d_dz, nf, c->d_g);
  dim3 const gb((kBtK * kBtN + 255) / 256, nf, b.n);
  if (tcp)
    tc_launch_btu(c->d_g, b.n, c->d_btu, false, nullptr, c->stream);
  else if (precision == HLBL_FP64)
    bt_build_kernel<double><<<gb, 256, 0, c->stream>>>(c->d_g, c->d_g + kGDzuLen, kGLen,
                                                       (size_t)nf * kGLen, nf, static_cast<double*>(c->d_bt));
  else
    bt_build_kernel<float><<<gb, 256, 0, c->stream>>>(c->d_g, c->d_g + kGDzuLen, kGLen,
                                                      (size_t)nf * kGLen, nf, static_cast<float*>(c->d_bt));
  return HLBL_OK;
}

// The QED weights of the batch's pairs into d_w ([pair][V][3][6]).
int run_weights(hlbl_ctx* c, const Geometry& geo, const PairBatch& b, double xunit, int precision) {
  long long const need = geo.V * b.n;
  if (need > c->w_cap) {
    if (c->capturing) return fail(HLBL_ESTATE, "QED weight buffer too small during graph capture");
    cudaFree(c->d_w);
    c->d_w = nullptr;
    c->w_cap = 0;
    cudaError_t e = cudaMalloc(&c->d_w, sizeof(double) * 3 * HLBL_QED_NW * (size_t)need);
    if (e != cudaSuccess) return fail(HLBL_ENOMEM, "QED weight buffer: %s", cudaGetErrorString(e));
    c->w_cap = need;
  }
  WArgs wa{};
  wa.batch = b;
  wa.xunit = xunit;
  wa.qp = c->qp;
  if (c->qed_mode == HLBL_QED_SURROGATE)
    return sur::launch_surrogate_weights(c->sur, geo, wa, c->sur_r0, c->qf, c->qed_fp32 ? c->qed_r64 : 1e300,
                                         c->d_w, c->d_fallback, c->stream, c->nsm);
  long long const n = geo.V * 3;
  int const blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)c->nsm * 16 / b.n));
  if (precision == HLBL_FP32 && c->qed_fp32) {
    // one thread per site (its three evaluations)
    int const bs = (int)std::max<long long>(1, std::min<long long>((geo.V + 255) / 256, (long long)c->nsm * 16 / b.n));
    qed_weights_fp32_kernel<<<dim3(bs, b.n), 256, 0, c->stream>>>(geo, wa, c->qed_r64, c->qf, c->d_w);
  } else {
    qed_weights_exact_kernel<<<dim3(blocks, b.n), 256, 0, c->stream>>>(geo, wa, c->d_w);
  }
  return HLBL_OK;
}

QedSel qed_sel(const hlbl_ctx* c) {
  QedSel q;
  q.kind = c->qed_kind;
  q.qp = c->qp;
  q.qf = c->qf;
  q.r64 = c->qed_fp32 ? c->qed_r64 : 1e300;  // the FP32 path's weight setting (hlbl_ctx_set_qed_fp32)
  q.t64 = c->d_dense64;
  q.t32 = c->d_dense32;
#ifdef HLBL_WITH_KQED
  q.kq = c->kq;
#endif
  return q;
}

// Bytes of the generic path's coefficients for n pairs.
size_t coef_bytes(const Geometry& geo, int n, bool f32) {
  return (size_t)n * (f32 ? sizeof(float) * coef32_per_pair(geo.V) : sizeof(double) * coef64_per_pair(geo.V));
}

int ensure_coef(hlbl_ctx* c, size_t need) {
  if (need <= c->coef_cap) return HLBL_OK;
  if (c->capturing) return fail(HLBL_ESTATE, "QED coefficient buffer too small during graph capture");
  cudaStreamSynchronize(c->stream);
  cudaFree(c->d_coef);
  c->d_coef = nullptr;
  c->coef_cap = 0;
  cudaError_t e = cudaMalloc(&c->d_coef, need);
  if (e != cudaSuccess) return fail(HLBL_ENOMEM, "QED coefficient buffer (%zu bytes): %s", need, cudaGetErrorString(e));
  c->coef_cap = need;
  return HLBL_OK;
}

// The QED weighting of pass 2 for the batch's pairs: the stand-in's weights
// (closed form) or the generic path's coefficients (FP32 layout for the
// FP32 path, FP64 layout for the FP64 path), recorded in a.
int run_qed(hlbl_ctx* c, const Geometry& geo, const PairBatch& b, double xunit, int precision, P2Args& a) {
  a.w = nullptr;
  a.coef = nullptr;
  a.coef_stride = 0;
  if (c->qed_kind == kQedStandInClosed) {
    if (int rc = run_weights(c, geo, b, xunit, precision)) return rc;
    a.w = c->d_w;
    return HLBL_OK;
  }
  bool const f32 = precision == HLBL_FP32;
  if (int rc = ensure_coef(c, coef_bytes(geo, b.n, f32))) return rc;
  if (int rc = coef_launch(qed_sel(c), f32, geo, b, xunit, c->d_coef, c->stream)) return rc;
  a.coef = c->d_coef;
  a.coef_stride = f32 ? coef32_per_pair(geo.V) : coef64_per_pair(geo.V);
  return HLBL_OK;
}

// Pass 2 for the batch's pairs with Bt already built; pair i's sums go to
// b.p[i].out[0..nf) (added if add).
int run_pass2(hlbl_ctx* c, const Geometry& geo, const double* y, const PairBatch& b, double xunit,
              int f0, int nf, int precision, int add) {
  P2Args a{};
  if (int rc = run_qed(c, geo, b, xunit, precision, a)) return rc;
  a.xunit = xunit;
  a.f0 = f0;
  int grid;
  prof_begin(c, 1);
  if (precision == HLBL_FP64) {
    const double* bt = static_cast<const double*>(c->d_bt);
    if (nf == 2) { grid = per_pair_grid(c->grid_p2d2, b.n, P2D2::tiles(geo.V)); P2D2::launch(grid, c->stream, y, b, geo, a, bt, c->d_part2, c->d_err); }
    else { grid = per_pair_grid(c->grid_p2d1, b.n, P2D1::tiles(geo.V)); P2D1::launch(grid, c->stream, y, b, geo, a, bt, c->d_part2, c->d_err); }
  } else if (use_tc(c, precision, nf)) {
    TcBatch tb{};
    tb.y32 = x32_block(c, geo, 0);
    for (int i = 0; i < b.n; ++i) {
      tb.x32[i] = x32_block(c, geo, 1 + i);
      for (int r = 0; r < 4; ++r) { tb.gsx[i][r] = b.p[i].gsx[r]; tb.yv[i][r] = b.p[i].yv[r]; }
    }
    grid = per_pair_grid(c->grid_tc, b.n, tc_tiles(geo.V));
    tc_launch_p2(grid, b.n, c->stream, tb, geo, a, c->d_btu, false, nullptr, c->d_part2, c->d_err);
  } else {
    const float* bt = static_cast<const float*>(c->d_bt);
    if (nf == 2 && c->p2_small) { grid = per_pair_grid(c->grid_p2f2s, b.n, P2F2s::tiles(geo.V)); P2F2s::launch(grid, c->stream, y, b, geo, a, bt, c->d_part2, c->d_err); }
    else if (nf == 2) { grid = per_pair_grid(c->grid_p2f2, b.n, P2F2::tiles(geo.V)); P2F2::launch(grid, c->stream, y, b, geo, a, bt, c->d_part2, c->d_err); }
    else { grid = per_pair_grid(c->grid_p2f1, b.n, P2F1::tiles(geo.V)); P2F1::launch(grid, c->stream, y, b, geo, a, bt, c->d_part2, c->d_err); }
  }
  prof_end(c, 1);
  p2_reduce_kernel<<<b.n, 64, 0, c->stream>>>(c->d_part2, grid, nf, b, add);
  return HLBL_OK;
}

// The FP32-copy path for one pair group: pass 1 on the copies, reduction,
// gamma insertion, the tensor-core B operand, the weights and the
// tensor-core pass 2 (b gives outputs and coordinates; tb the copies).
int run_group_f32(hlbl_ctx* c, const PairBatch& b, const TcBatch& tb, double xunit) {
  if (c->stage_pending) {
    cudaError_t e = cudaStreamWaitEvent(c->stream, c->stage_ev, 0);
    if (e != cudaSuccess) return cuda_fail(e, "wait for staged block");
    c->stage_pending = false;
  }
  Geometry const& geo = c->geo;
  int const v = c->p1f_var;
  int const g1 = per_pair_grid(c->grid_p1f[v], b.n, p1f32_tiles(geo.V));
  prof_begin(c, 0);
  p1f32_launch(v, g1, b.n, c->stream, tb, geo, c->d_part1, c->d_err);
  prof_end(c, 0);
  p1_reduce_kernel<<<dim3((kDzLen + kRedOut - 1) / kRedOut, 2, b.n), kRedOut * kRedGrp, 0, c->stream>>>(c->d_part1, g1, 2, c->d_dz,
                                                                             nullptr, nullptr);
  g_build_kernel<<<dim3((kGLen / 2 + 255) / 256, 2, b.n), 256, 0, c->stream>>>(c->d_dz, 2, c->d_g);
  tc_launch_btu(c->d_g, b.n, c->d_btu, c->tc16 != 0, c->d_bscale, c->stream);
  P2Args a{};
  if (int rc = run_qed(c, geo, b, xunit, HLBL_FP32, a)) return rc;
  a.xunit = xunit;
  a.f0 = 0;
  int const g2 = per_pair_grid(c->grid_tc, b.n, tc_tiles(geo.V));
  prof_begin(c, 1);
  tc_launch_p2(g2, b.n, c->stream, tb, geo, a, c->d_btu, c->tc16 != 0, c->d_bscale, c->d_part2, c->d_err);
  prof_end(c, 1);
  p2_reduce_kernel<<<b.n, 64, 0, c->stream>>>(c->d_part2, g2, 2, b, 0);
  return HLBL_OK;
}

PairBatch one_pair(const double* src, double* out, const int gsx[4], const int yv[4]) {
  PairBatch b{};
  b.n = 1;
  b.p[0].src = src;
  b.p[0].out = out;
  for (int r = 0; r < 4; ++r) {
    b.p[0].gsx[r] = gsx[r];
    b.p[0].yv[r] = yv ? yv[r] : 0;
  }
  return b;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return HLBL_OK;
}

}  // namespace hg

extern "C" {

const char* hlbl_last_error(void) { return g_last_error.c_str(); }
const char* hlbl_version(void) { return "hlbl_gb300 0.1 (sm_103a)"; }

uint64_t hlbl_source_seed(uint64_t run_seed, const int gsx[4]) {
  return hlbl_rng_source_seed(run_seed, gsx);
}

int hlbl_ctx_create(hlbl_ctx** out, const int global[4], const int local[4],
                    const int proc_coords[4], double lambda, int device) {
  if (!out || !global || !local || !proc_coords) return fail(HLBL_EINVAL, "hlbl_ctx_create: null argument");
  *out = nullptr;
  Geometry geo{};
  if (int rc = make_geometry(global, local, proc_coords, geo)) return rc;
  if (!(lambda > 0)) return fail(HLBL_EINVAL, "hlbl_ctx_create: lambda must be positive");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  hlbl_ctx* c = new hlbl_ctx();
  c->device = device;
  c->geo = geo;
  hlbl_qed_params_init(&c->qp, lambda);
  qed_f32_tables(c->qp, c->qf);
  auto bail = [&](int rc) { hlbl_ctx_destroy(c); return rc; };
  e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return bail(cuda_fail(e, "SM count"));
  int rc;
  if ((rc = P1D2::init(c->nsm, c->grid_p1d2)) || (rc = P1D1::init(c->nsm, c->grid_p1d1)) ||
      (rc = P1F2::init(c->nsm, c->grid_p1f2)) || (rc = P1F1::init(c->nsm, c->grid_p1f1)) ||
      (rc = P2D2::init(c->nsm, c->grid_p2d2)) || (rc = P2D1::init(c->nsm, c->grid_p2d1)) ||
      (rc = P2F2::init(c->nsm, c->grid_p2f2)) || (rc = P2F1::init(c->nsm, c->grid_p2f1)) ||
      (rc = P1F2s::init(c->nsm, c->grid_p1f2s)) || (rc = P2F2s::init(c->nsm, c->grid_p2f2s)) ||
      (rc = tc_init(c->nsm, c->grid_tc)) || (rc = p1f32_init(c->nsm, c->grid_p1f)) ||
      (rc = coef_init(c->nsm)))
    return bail(rc);
  c->max_grid = std::max({c->grid_p1d2, c->grid_p1d1, c->grid_p1f2, c->grid_p1f1, c->grid_p2d2,
                          c->grid_p2d1, c->grid_p2f2, c->grid_p2f1, c->grid_p1f2s, c->grid_p2f2s,
                          c->grid_tc, c->grid_p1f[0], c->grid_p1f[1], c->grid_p1f[2], c->grid_p1f[3]});
  e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->stage_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->compute_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(cuda_fail(e, "copy stream"));
  e = cudaStreamCreate(&c->own_stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
  c->stream = c->own_stream;
  // per-pair work buffers for up to kMaxBatch pairs; the partial sums of a
  // batch never exceed max(resident grid, kMaxBatch) thread blocks
  size_t const slots = (size_t)std::max(c->max_grid, kMaxBatch);
  struct { void** p; size_t n; } bufs[] = {
      {(void**)&c->d_part1, sizeof(double) * slots * 2 * kDzLen},
      {(void**)&c->d_part2, sizeof(double) * slots * 2},
      {(void**)&c->d_dz, sizeof(double) * kMaxBatch * 2 * kDzLen},
      {(void**)&c->d_g, sizeof(double) * kMaxBatch * 2 * kGLen},
      {(void**)&c->d_bt, sizeof(double) * kMaxBatch * 2 * kBtK * kBtN},
      {(void**)&c->d_btu, sizeof(float) * kMaxBatch * tc_btu_floats_per_pair()},
      {(void**)&c->d_bscale, sizeof(float) * kMaxBatch * 2},
      {(void**)&c->d_out, sizeof(double) * 2},
      {(void**)&c->d_err, sizeof(int)}};
  for (auto& b : bufs) {
    e = cudaMalloc(b.p, b.n);
    if (e != cudaSuccess) return bail(fail(HLBL_ENOMEM, "cudaMalloc %zu bytes: %s", b.n, cudaGetErrorString(e)));
  }
  e = cudaMemset(c->d_err, 0, sizeof(int));
  if (e != cudaSuccess) return bail(cuda_fail(e, "error flag"));
  e = cudaMallocHost(reinterpret_cast<void**>(&c->h_out), sizeof(double) * 2);
  if (e != cudaSuccess) return bail(fail(HLBL_ENOMEM, "cudaMallocHost: %s", cudaGetErrorString(e)));
  *out = c;
  return HLBL_OK;
}

void hlbl_ctx_destroy(hlbl_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->own_stream) cudaStreamSynchronize(c->own_stream);
  cudaFree(c->d_part1);
  cudaFree(c->d_part2);
  cudaFree(c->d_dz);
  cudaFree(c->d_g);
  cudaFree(c->d_bt);
  cudaFree(c->d_btu);
  cudaFree(c->d_bscale);
  cudaFree(c->d_x32);
  cudaFree(c->d_out);
  cudaFree(c->d_err);
  cudaFree(c->d_w);
  cudaFree(c->d_coef);
  cudaFree(c->d_dense64);
  cudaFree(c->d_dense32);
  cudaFree(c->d_fallback);
  cudaFree(c->d_p22_out);
  p22_destroy(c->p22);
  if (c->h_out) cudaFreeHost(c->h_out);
  for (auto& pe : c->ev)
    for (auto& e : pe)
      if (e) cudaEventDestroy(e);
  if (c->copy_stream) { cudaStreamSynchronize(c->copy_stream); cudaStreamDestroy(c->copy_stream); }
  if (c->stage_ev) cudaEventDestroy(c->stage_ev);
  if (c->compute_ev) cudaEventDestroy(c->compute_ev);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

int hlbl_selftest_wait_timeout(hlbl_ctx* c) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_selftest_wait_timeout: null context");
  wait_timeout_selftest_kernel<<<1, 32, 0, c->stream>>>(c->d_err);
  return check_launch("hlbl_selftest_wait_timeout launch");
}

int hlbl_ctx_check(hlbl_ctx* c) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_check: null context");
  int flag = 0;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(&flag, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_ctx_check");
  if (flag) {
    cudaMemset(c->d_err, 0, sizeof(int));
    return fail(HLBL_ECUDA, "a contraction kernel gave up waiting for its staged tile (code %d); "
                            "the sums since the last check are invalid", flag);
  }
  return HLBL_OK;
}

int hlbl_ctx_set_stream(hlbl_ctx* c, void* stream) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_stream: null context");
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return HLBL_OK;
}

size_t hlbl_block_length(const hlbl_ctx* c) { return c ? (size_t)c->geo.V * 2 * 12 * 24 : 0; }

int hlbl_kernel_sum_async(hlbl_ctx* c, const double* src, const double* y, const int gsx[4],
                          const int yv[4], double xunit, int precision, double* d_out) {
  if (!c || !src || !y || !gsx || !yv || !d_out) return fail(HLBL_EINVAL, "hlbl_kernel_sum: null argument");
  if (!aligned16(src) || !aligned16(y)) return fail(HLBL_EINVAL, "hlbl_kernel_sum: blocks must be 16-byte aligned");
  if (precision != HLBL_FP64 && precision != HLBL_FP32) return fail(HLBL_EINVAL, "hlbl_kernel_sum: bad precision %d", precision);
  for (int r = 0; r < 4; ++r)
    if (gsx[r] < 0 || gsx[r] >= c->geo.global[r]) return fail(HLBL_EINVAL, "hlbl_kernel_sum: gsx[%d] = %d outside [0, %d)", r, gsx[r], c->geo.global[r]);
  PairBatch const b = one_pair(src, d_out, gsx, yv);
  if (int rc = run_pass1(c, c->geo, y, b, 0, 2, precision, nullptr, nullptr, true)) return rc;
  if (int rc = run_pass2(c, c->geo, y, b, xunit, 0, 2, precision, 0)) return rc;
  return check_launch("hlbl_kernel_sum launch");
}

size_t hlbl_f32_block_length(const hlbl_ctx* c) { return c ? f32_block_floats(c->geo.V) : 0; }

int hlbl_kernel_sums_batched_f32(hlbl_ctx* c, const float* y32, int n, const float* const* x32s,
                                 const int* gsx, const int* yv, double xunit, double* d_out) {
  if (!c || !y32 || !x32s || !gsx || !yv || !d_out || n < 0)
    return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched_f32: bad argument");
  if (!aligned16(y32)) return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched_f32: copies must be 16-byte aligned");
  for (int i = 0; i < n; ++i) {
    if (!x32s[i] || !aligned16(x32s[i]))
      return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched_f32: copy %d null or not 16-byte aligned", i);
    for (int r = 0; r < 4; ++r)
      if (gsx[4 * i + r] < 0 || gsx[4 * i + r] >= c->geo.global[r])
        return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched_f32: gsx of pair %d outside the lattice", i);
  }
  int const group = c->group_f32 > 0 ? std::min(c->group_f32, kMaxBatch) : kMaxBatch;
  if (c->capturing) {
    bool const small = c->qed_kind == kQedStandInClosed
                           ? c->geo.V * std::min(std::max(n, 1), kMaxBatch) > c->w_cap
                           : coef_bytes(c->geo, std::min(std::max(n, 1), group), true) > c->coef_cap;
    if (small) return fail(HLBL_ESTATE, "QED weight buffer too small during graph capture");
  }
  for (int i0 = 0; i0 < n; i0 += group) {
    PairBatch b{};
    TcBatch tb{};
    b.n = std::min(group, n - i0);
    tb.y32 = y32;
    for (int i = 0; i < b.n; ++i) {
      b.p[i].out = d_out + 2 * (size_t)(i0 + i);
      tb.x32[i] = x32s[i0 + i];
      for (int r = 0; r < 4; ++r) {
        b.p[i].gsx[r] = tb.gsx[i][r] = gsx[4 * (i0 + i) + r];
        b.p[i].yv[r] = tb.yv[i][r] = yv[4 * (i0 + i) + r];
      }
    }
    if (int rc = run_group_f32(c, b, tb, xunit)) return rc;
  }
  return check_launch("hlbl_kernel_sums_batched_f32 launch");
}

int hlbl_autotune_f32(hlbl_ctx* c, const float* y32, int n, const float* const* x32s, const int* gsx,
                      const int* yv, double xunit, double* d_out, int* best_variant, int* best_group,
                      double* best_ms) {
  if (!c || n < 1) return fail(HLBL_EINVAL, "hlbl_autotune_f32: bad argument");
  if (int rc = hlbl_ctx_reserve(c, n)) return rc;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 1e300;
  int bv = 1, bg = 1;
  int const groups[] = {1, 2, 4, 8, 16};
  for (int v = 0; v < kP1f32Variants; ++v)
    for (int g : groups) {
      if (g > 1 && g / 2 >= n) continue;
      c->p1f_var = v;
      c->group_f32 = g;
      cudaEventRecord(a, c->stream);
      int rc = hlbl_kernel_sums_batched_f32(c, y32, n, x32s, gsx, yv, xunit, d_out);
      cudaEventRecord(b, c->stream);
      cudaError_t e = cudaEventSynchronize(b);
      if (rc || e != cudaSuccess) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return rc ? rc : cuda_fail(e, "hlbl_autotune_f32");
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (ms < best) { best = ms; bv = v; bg = g; }
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  c->p1f_var = bv;
  c->group_f32 = bg;
  if (best_variant) *best_variant = bv;
  if (best_group) *best_group = bg;
  if (best_ms) *best_ms = best;
  return HLBL_OK;
}

int hlbl_kernel_sums_batched(hlbl_ctx* c, const double* y, int n, const double* const* srcs,
                             const int* gsx, const int* yv, double xunit, int precision,
                             double* d_out) {
  if (!c || !y || !srcs || !gsx || !yv || !d_out || n < 0)
    return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched: bad argument");
  if (precision != HLBL_FP64 && precision != HLBL_FP32)
    return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched: bad precision %d", precision);
  if (!aligned16(y)) return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched: blocks must be 16-byte aligned");
  for (int i = 0; i < n; ++i) {
    if (!srcs[i] || !aligned16(srcs[i]))
      return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched: block %d null or not 16-byte aligned", i);
    for (int r = 0; r < 4; ++r)
      if (gsx[4 * i + r] < 0 || gsx[4 * i + r] >= c->geo.global[r])
        return fail(HLBL_EINVAL, "hlbl_kernel_sums_batched: gsx of pair %d outside the lattice", i);
  }
  int const group = c->batch_group > 0 ? std::min(c->batch_group, kMaxBatch) : kMaxBatch;
  for (int i0 = 0; i0 < n; i0 += group) {
    PairBatch b{};
    b.n = std::min(group, n - i0);
    for (int i = 0; i < b.n; ++i) {
      b.p[i].src = srcs[i0 + i];
      b.p[i].out = d_out + 2 * (size_t)(i0 + i);
      for (int r = 0; r < 4; ++r) {
        b.p[i].gsx[r] = gsx[4 * (i0 + i) + r];
        b.p[i].yv[r] = yv[4 * (i0 + i) + r];
      }
    }
    if (int rc = run_pass1(c, c->geo, y, b, 0, 2, precision, nullptr, nullptr, true)) return rc;
    if (int rc = run_pass2(c, c->geo, y, b, xunit, 0, 2, precision, 0)) return rc;
  }
  return check_launch("hlbl_kernel_sums_batched launch");
}

int hlbl_f32_tile_copy(hlbl_ctx* c, const double* d_block, float* d_out) {
  if (!c || !d_block || !d_out) return fail(HLBL_EINVAL, "hlbl_f32_tile_copy: null argument");
  if (!aligned16(d_block) || !aligned16(d_out)) return fail(HLBL_EINVAL, "hlbl_f32_tile_copy: pointers must be 16-byte aligned");
  if (c->stage_pending) {  // a block staged on the side stream must have landed
    cudaError_t e = cudaStreamWaitEvent(c->stream, c->stage_ev, 0);
    if (e != cudaSuccess) return cuda_fail(e, "wait for staged block");
    c->stage_pending = false;
  }
  cudaError_t e = cudaMemsetAsync(d_out + f32_tile_floats(c->geo.V), 0, kF32Trailer * sizeof(float), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_f32_tile_copy trailer");
  f32_tile_copy_kernel<<<dim3(std::max(1, c->nsm * 8 / 24), 24), 256, 0, c->stream>>>(d_block, c->geo, d_out);
  return check_launch("hlbl_f32_tile_copy launch");
}

int hlbl_ctx_set_tc_fp16(hlbl_ctx* c, int on) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_tc_fp16: null context");
  c->tc16 = on ? 1 : 0;
  return HLBL_OK;
}

int hlbl_ctx_set_qed_fp32(hlbl_ctx* c, int on, double r64) {
  if (!c || !(r64 >= 0)) return fail(HLBL_EINVAL, "hlbl_ctx_set_qed_fp32: bad argument");
  c->qed_fp32 = on ? 1 : 0;
  c->qed_r64 = r64;
  return HLBL_OK;
}

int hlbl_ctx_set_p1f32_variant(hlbl_ctx* c, int variant, int group) {
  if (!c || variant < 0 || variant >= kP1f32Variants || group < 0 || group > kMaxBatch)
    return fail(HLBL_EINVAL, "hlbl_ctx_set_p1f32_variant: bad argument");
  c->p1f_var = variant;
  c->group_f32 = group;
  return HLBL_OK;
}

int hlbl_ctx_set_tensor_cores(hlbl_ctx* c, int on) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_tensor_cores: null context");
  c->tc = on ? 1 : 0;
  return HLBL_OK;
}

int hlbl_ctx_set_batch_group(hlbl_ctx* c, int group) {
  if (!c || group < 0) return fail(HLBL_EINVAL, "hlbl_ctx_set_batch_group: bad argument");
  c->batch_group = group;
  return HLBL_OK;
}

int hlbl_kernel_sum(hlbl_ctx* c, const double* src, const double* y, const int gsx[4],
                    const int yv[4], double xunit, int precision, double out[2]) {
  if (!out) return fail(HLBL_EINVAL, "hlbl_kernel_sum: null out");
  if (int rc = hlbl_kernel_sum_async(c, src, y, gsx, yv, xunit, precision, c ? c->d_out : nullptr)) return rc;
  cudaError_t e = cudaMemcpyAsync(c->h_out, c->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "result copy");
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_kernel_sum");
  if (int rc = hlbl_ctx_check(c)) return rc;
  out[0] = c->h_out[0];
  out[1] = c->h_out[1];
  return HLBL_OK;
}

int hlbl_cu_dzu_dzsu(hlbl_ctx* c, double* d_dzu, double* d_dzsu, const double* src,
                     const double* y, int iflavor, const int pc[4], const int gsx[4],
                     const int global[4], const int local[4]) {
  if (!c || !d_dzu || !d_dzsu || !src || !y) return fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu: null argument");
  if (iflavor != 0 && iflavor != 1) return fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu: iflavor must be 0 or 1");
  if (!aligned16(src) || !aligned16(y)) return fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu: blocks must be 16-byte aligned");
  Geometry geo{};
  if (int rc = make_geometry(global, local, pc, geo)) return rc;
  PairBatch const b = one_pair(src, nullptr, gsx, nullptr);
  if (int rc = run_pass1(c, geo, y, b, iflavor, 1, HLBL_FP64, d_dzu, d_dzsu, false)) return rc;
  return check_launch("hlbl_cu_dzu_dzsu launch");
}

int hlbl_insert_gammas(hlbl_ctx* c, const double* d_dzu, const double* d_dzsu, double* d_g_dzu,
                       double* d_g_dzsu) {
  if (!c || !d_dzu || !d_dzsu || !d_g_dzu || !d_g_dzsu) return fail(HLBL_EINVAL, "hlbl_insert_gammas: null argument");
  cudaError_t e = cudaMemcpyAsync(c->d_dz, d_dzu, kDzuLen * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_dz + kDzuLen, d_dzsu, (kDzLen - kDzuLen) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_insert_gammas copy");
  g_build_kernel<<<dim3((kGLen / 2 + 255) / 256, 1, 1), 256, 0, c->stream>>>(c->d_dz, 1, c->d_g);
  e = cudaMemcpyAsync(d_g_dzu, c->d_g, kGDzuLen * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_g_dzsu, c->d_g + kGDzuLen, (kGLen - kGDzuLen) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_insert_gammas copy");
  return check_launch("hlbl_insert_gammas launch");
}

int hlbl_cu_4pt_contraction(hlbl_ctx* c, double* d_ks, const double* d_g_dzu,
                            const double* d_g_dzsu, const double* src, const double* y,
                            int iflavor, const int pc[4], const int gsx[4], double xunit,
                            const int yv[4], const int global[4], const int local[4]) {
  if (!c || !d_ks || !d_g_dzu || !d_g_dzsu || !src || !y) return fail(HLBL_EINVAL, "hlbl_cu_4pt_contraction: null argument");
  if (iflavor != 0 && iflavor != 1) return fail(HLBL_EINVAL, "hlbl_cu_4pt_contraction: iflavor must be 0 or 1");
  if (!aligned16(src) || !aligned16(y)) return fail(HLBL_EINVAL, "hlbl_cu_4pt_contraction: blocks must be 16-byte aligned");
  Geometry geo{};
  if (int rc = make_geometry(global, local, pc, geo)) return rc;
  bt_build_kernel<double><<<dim3((kBtK * kBtN + 255) / 256, 1, 1), 256, 0, c->stream>>>(
      d_g_dzu, d_g_dzsu, 0, 0, 1, static_cast<double*>(c->d_bt));
  PairBatch const b = one_pair(src, d_ks, gsx, yv);
  if (int rc = run_pass2(c, geo, y, b, xunit, iflavor, 1, HLBL_FP64, 1)) return rc;
  return check_launch("hlbl_cu_4pt_contraction launch");
}

// ---- 2+2 pieces (pieces_2p2.cu) -----------------------------------------

int hlbl_2p2_lmax(const hlbl_ctx* c) { return c ? p22_lmax(c->geo) : 0; }

int hlbl_ctx_set_2p2_r64(hlbl_ctx* c, double r64) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_2p2_r64: null context");
  if (!(r64 >= 0.0)) return fail(HLBL_EINVAL, "hlbl_ctx_set_2p2_r64: r64 = %g", r64);
  c->p22_r64 = r64;
  return HLBL_OK;
}

int hlbl_2p2_reserve(hlbl_ctx* c) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_2p2_reserve: null context");
  return p22_reserve(&c->p22, c->geo, c->nsm);
}

static int p22_args(hlbl_ctx* c, const char* what, const double* fwd, int iflavor, const int gsw[4],
                    const int* targets, int n_y, int precision) {
  if (!c || !fwd || !gsw || (n_y > 0 && !targets)) return fail(HLBL_EINVAL, "%s: null argument", what);
  if (!aligned16(fwd)) return fail(HLBL_EINVAL, "%s: block must be 16-byte aligned", what);
  if (iflavor != 0 && iflavor != 1) return fail(HLBL_EINVAL, "%s: iflavor must be 0 or 1", what);
  if (n_y < 0) return fail(HLBL_EINVAL, "%s: n_y = %d", what, n_y);
  if (precision != HLBL_FP64 && precision != HLBL_FP32) return fail(HLBL_EINVAL, "%s: bad precision %d", what, precision);
  for (int r = 0; r < 4; ++r)
    if (gsw[r] < 0 || gsw[r] >= c->geo.global[r])
      return fail(HLBL_EINVAL, "%s: gsw[%d] = %d outside [0, %d)", what, r, gsw[r], c->geo.global[r]);
  for (int t = 0; t < n_y; ++t)
    for (int r = 0; r < 4; ++r)
      if (targets[4 * t + r] < 0 || targets[4 * t + r] >= c->geo.global[r])
        return fail(HLBL_EINVAL, "%s: target %d coordinate %d = %d outside [0, %d)", what, t, r,
                    targets[4 * t + r], c->geo.global[r]);
  return HLBL_OK;
}

static int p22_launch(hlbl_ctx* c, const double* fwd, int iflavor, const int gsw[4], const int* targets,
                      int n_y, double xunit, int precision, double* d_p1, double* d_p234, int raw,
                      const float* x32 = nullptr) {
  P22Request rq{};
  rq.fwd = fwd;
  rq.x32 = x32;
  rq.iflavor = iflavor;
  for (int r = 0; r < 4; ++r) rq.gsw[r] = gsw[r];
  rq.targets = targets;
  rq.n_y = n_y;
  rq.xunit = xunit;
  rq.precision = precision;
  rq.r64 = c->p22_r64;
  rq.d_p1 = d_p1;
  rq.d_p234 = d_p234;
  rq.raw_layout = raw;
  if (int rc = p22_run(&c->p22, c->stream, c->geo, qed_sel(c), c->nsm, c->capturing, rq)) return rc;
  return check_launch("2+2 launch");
}

int hlbl_pieces_2p2_async(hlbl_ctx* c, const double* d_fwd, const int gsw[4], const int* targets, int n_y,
                          double xunit, int precision, double* d_p1, double* d_p234) {
  if (int rc = p22_args(c, "hlbl_pieces_2p2_async", d_fwd, 0, gsw, targets, n_y, precision)) return rc;
  if (!d_p1 || (n_y > 0 && !d_p234)) return fail(HLBL_EINVAL, "hlbl_pieces_2p2_async: null output");
  return p22_launch(c, d_fwd, 0, gsw, targets, n_y, xunit, precision, d_p1, d_p234, 0);
}

int hlbl_pieces_2p2_f32(hlbl_ctx* c, const float* d_x32, const int gsw[4], const int* targets, int n_y,
                        double xunit, double* d_p1, double* d_p234) {
  // the argument checks of the FP64-block call, on the copy's address
  if (int rc = p22_args(c, "hlbl_pieces_2p2_f32", reinterpret_cast<const double*>(d_x32), 0, gsw, targets, n_y,
                        HLBL_FP32))
    return rc;
  if (!d_p1 || (n_y > 0 && !d_p234)) return fail(HLBL_EINVAL, "hlbl_pieces_2p2_f32: null output");
  return p22_launch(c, nullptr, 0, gsw, targets, n_y, xunit, HLBL_FP32, d_p1, d_p234, 0, d_x32);
}

// the blocking calls: results on the device, then copied to the host arrays
static int p22_blocking(hlbl_ctx* c, const double* fwd, int iflavor, const int gsw[4], const int* targets,
                        int n_y, double xunit, int precision, double* p1, double* p234, int raw) {
  if (!p1 || (n_y > 0 && !p234)) return fail(HLBL_EINVAL, "2+2: null output");
  size_t const n1 = (size_t)64 * p22_lmax(c->geo), n234 = (size_t)n_y * 5 * 64;
  if (c->p22_out_cap < n1 + n234) {
    cudaFree(c->d_p22_out);
    c->d_p22_out = nullptr;
    c->p22_out_cap = 0;
    cudaError_t e = cudaMalloc(&c->d_p22_out, (n1 + n234) * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "2+2 results");
    c->p22_out_cap = n1 + n234;
  }
  if (int rc = p22_launch(c, fwd, iflavor, gsw, targets, n_y, xunit, precision, c->d_p22_out,
                          c->d_p22_out + n1, raw))
    return rc;
  cudaError_t e = cudaMemcpyAsync(p1, c->d_p22_out, n1 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && n234)
    e = cudaMemcpyAsync(p234, c->d_p22_out + n1, n234 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "2+2 result copy");
  return hlbl_ctx_check(c);
}

int hlbl_pieces_2p2(hlbl_ctx* c, const double* d_fwd, const int gsw[4], const int* targets, int n_y,
                    double xunit, int precision, double* p1, double* p234) {
  if (int rc = p22_args(c, "hlbl_pieces_2p2", d_fwd, 0, gsw, targets, n_y, precision)) return rc;
  return p22_blocking(c, d_fwd, 0, gsw, targets, n_y, xunit, precision, p1, p234, 0);
}

int hlbl_compute_2p2(hlbl_ctx* c, const double* d_fwd_y, double* P1, double* P234, int iflavor,
                     const int gsw[4], const int* gycoords, int n_y, double xunit, int precision) {
  if (int rc = p22_args(c, "hlbl_compute_2p2", d_fwd_y, iflavor, gsw, gycoords, n_y, precision)) return rc;
  return p22_blocking(c, d_fwd_y, iflavor, gsw, gycoords, n_y, xunit, precision, P1, P234, 1);
}

int hlbl_reserve_kernel_memory(hlbl_ctx* c, size_t* bytes) {
  if (!c || !bytes) return fail(HLBL_EINVAL, "hlbl_reserve_kernel_memory: null argument");
  size_t free0 = 0, free1 = 0, total = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemGetInfo(&free0, &total);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_reserve_kernel_memory");
  {
    int const tiny[4] = {2, 2, 2, 2}, zero[4] = {0, 0, 0, 0}, one[4] = {1, 1, 1, 1};
    Geometry geo{};
    make_geometry(tiny, tiny, zero, geo);
    double* blk = nullptr;
    size_t const n = (size_t)geo.V * 2 * 12 * 24;
    e = cudaMalloc(&blk, n * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "hlbl_reserve_kernel_memory alloc");
    cudaMemsetAsync(blk, 0, n * sizeof(double), c->stream);
    for (int prec : {HLBL_FP64, HLBL_FP32}) {
      for (int nf : {1, 2}) {
        PairBatch const b = one_pair(blk, c->d_out, zero, one);
        run_pass1(c, geo, blk, b, 0, nf, prec, nullptr, nullptr, true);
        run_pass2(c, geo, blk, b, 1.0, 0, nf, prec, 0);
      }
    }
    e = cudaStreamSynchronize(c->stream);
    cudaFree(blk);
    if (e != cudaSuccess) return cuda_fail(e, "hlbl_reserve_kernel_memory run");
  }
  e = cudaMemGetInfo(&free1, &total);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_reserve_kernel_memory");
  *bytes = free0 > free1 ? free0 - free1 : 0;
  return HLBL_OK;
}

int hlbl_ctx_reserve(hlbl_ctx* c, int max_pairs) {
  if (!c || max_pairs < 1) return fail(HLBL_EINVAL, "hlbl_ctx_reserve: bad argument");
  if (c->tc) {
    int const group = c->batch_group > 0 ? std::min(c->batch_group, kMaxBatch) : kMaxBatch;
    if (int rc = ensure_x32(c, c->geo, std::min(max_pairs, group))) return rc;
  }
  if (c->qed_kind != kQedStandInClosed) {
    // the generic path's coefficients: FP64 layout for the pair groups of the
    // FP64-block calls, FP32 layout for those of the FP32-copy path
    int const g64 = c->batch_group > 0 ? std::min(c->batch_group, kMaxBatch) : kMaxBatch;
    int const g32 = c->group_f32 > 0 ? std::min(c->group_f32, kMaxBatch) : kMaxBatch;
    return ensure_coef(c, std::max(coef_bytes(c->geo, std::min(max_pairs, g64), false),
                                   coef_bytes(c->geo, std::min(max_pairs, g32), true)));
  }
  long long const need = c->geo.V * std::min(max_pairs, kMaxBatch);
  if (need <= c->w_cap) return HLBL_OK;
  cudaStreamSynchronize(c->stream);
  cudaFree(c->d_w);
  c->d_w = nullptr;
  c->w_cap = 0;
  cudaError_t e = cudaMalloc(&c->d_w, sizeof(double) * 3 * HLBL_QED_NW * (size_t)need);
  if (e != cudaSuccess) return fail(HLBL_ENOMEM, "QED weight buffer: %s", cudaGetErrorString(e));
  c->w_cap = need;
  return HLBL_OK;
}

int hlbl_stage_async(hlbl_ctx* c, void* d_dst, const void* h_src, size_t bytes, int after_compute) {
  if (!c || !d_dst || !h_src) return fail(HLBL_EINVAL, "hlbl_stage_async: null argument");
  cudaError_t e = cudaSuccess;
  if (after_compute) {
    // the destination may still be read by contraction work already enqueued
    e = cudaEventRecord(c->compute_ev, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->compute_ev, 0);
    if (e != cudaSuccess) return cuda_fail(e, "hlbl_stage_async ordering");
  }
  e = cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, c->copy_stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->stage_ev, c->copy_stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_stage_async");
  c->stage_pending = true;
  return HLBL_OK;
}

int hlbl_autotune(hlbl_ctx* c, const double* y, int n, const double* const* srcs, const int* gsx,
                  const int* yv, double xunit, double* d_out, int* best_p1, int* best_p2,
                  int* best_group, double* best_ms) {
  if (!c || n < 1) return fail(HLBL_EINVAL, "hlbl_autotune: bad argument");
  if (int rc = hlbl_ctx_reserve(c, n)) return rc;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 1e300;
  int bp1 = 0, bp2 = 0, bg = kMaxBatch;
  int const groups[] = {1, 2, 4, 8, 16};
  for (int p1 = 0; p1 < 2; ++p1)
    for (int p2 = 0; p2 < 3; ++p2)
      for (int g : groups) {
        if (g > 1 && g / 2 >= n) continue;
        c->p1_small = p1;
        c->p2_small = p2 == 1;
        c->tc = p2 == 2;
        c->batch_group = g;
        if (c->tc)
          if (int rc = ensure_x32(c, c->geo, std::min(g, n))) {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            return rc;
          }
        cudaEventRecord(a, c->stream);
        int rc = hlbl_kernel_sums_batched(c, y, n, srcs, gsx, yv, xunit, HLBL_FP32, d_out);
        cudaEventRecord(b, c->stream);
        cudaError_t e = cudaEventSynchronize(b);
        if (rc || e != cudaSuccess) {
          cudaEventDestroy(a);
          cudaEventDestroy(b);
          return rc ? rc : cuda_fail(e, "hlbl_autotune");
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) { best = ms; bp1 = p1; bp2 = p2; bg = g; }
      }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  c->p1_small = bp1;
  c->p2_small = bp2 == 1;
  c->tc = bp2 == 2;
  c->batch_group = bg;
  if (best_p1) *best_p1 = bp1;
  if (best_p2) *best_p2 = bp2;
  if (best_group) *best_group = bg;
  if (best_ms) *best_ms = best;
  return HLBL_OK;
}

struct hlbl_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
};

int hlbl_graph_begin(hlbl_ctx* c) {
  if (!c || c->capturing) return fail(HLBL_ESTATE, "hlbl_graph_begin: no context or already capturing");
  if (int rc = hlbl_ctx_reserve(c, kMaxBatch)) return rc;
  if (c->stage_pending) {
    cudaError_t e = cudaStreamWaitEvent(c->stream, c->stage_ev, 0);
    if (e != cudaSuccess) return cuda_fail(e, "hlbl_graph_begin");
    c->stage_pending = false;
  }
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  c->capturing = true;
  return HLBL_OK;
}

int hlbl_graph_end(hlbl_ctx* c, hlbl_graph** out) {
  if (!c || !out || !c->capturing) return fail(HLBL_ESTATE, "hlbl_graph_end: not capturing");
  c->capturing = false;
  hlbl_graph* g = new hlbl_graph();
  cudaError_t e = cudaStreamEndCapture(c->stream, &g->graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(e, "hlbl_graph_end");
  }
  g->stream = c->stream;
  *out = g;
  return HLBL_OK;
}

int hlbl_graph_launch(hlbl_graph* g, void* stream) {
  if (!g) return fail(HLBL_EINVAL, "hlbl_graph_launch: null graph");
  cudaError_t e = cudaGraphLaunch(g->exec, stream ? static_cast<cudaStream_t>(stream) : g->stream);
  return e == cudaSuccess ? HLBL_OK : cuda_fail(e, "cudaGraphLaunch");
}

void hlbl_graph_destroy(hlbl_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

int hlbl_ctx_set_qed_kernel(hlbl_ctx* c, int kind, uint64_t seed) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_qed_kernel: null context");
  if (kind < 0 || kind >= kQedKinds) return fail(HLBL_EINVAL, "hlbl_ctx_set_qed_kernel: bad kind %d", kind);
#ifdef HLBL_WITH_KQED
  if (kind == kQedKqed && !c->kq_ready) {
    // KQED's host set-up (bin/hlbl_hypercube.cpp:174-178), once per context
    if (initialise(&c->kq) != 0) return fail(HLBL_ECUDA, "hlbl_ctx_set_qed_kernel: KQED initialise failed");
    c->kq_ready = true;
  }
#else
  if (kind == kQedKqed)
    return fail(HLBL_EINVAL, "hlbl_ctx_set_qed_kernel: this library was built without KQED (HLBL_KQED_DIR)");
#endif
  if (c->capturing) return fail(HLBL_ESTATE, "hlbl_ctx_set_qed_kernel: during graph capture");
  if (kind != kQedStandInClosed && c->qed_mode == HLBL_QED_SURROGATE)
    return fail(HLBL_ESTATE, "hlbl_ctx_set_qed_kernel: the learned weight replaces the stand-in's closed form only");
  if (kind == kQedDense || kind == kQedDenseKerv) {
    std::vector<double> t64((size_t)HLBL_QED_DENSE_NB * HLBL_QED_NK);
    hlbl_qed_dense_init(t64.data(), (unsigned long long)seed);
    std::vector<float> t32(t64.size());
    for (size_t i = 0; i < t64.size(); ++i) t32[i] = (float)t64[i];
    cudaError_t e = cudaSuccess;
    if (!c->d_dense64) e = cudaMalloc(&c->d_dense64, sizeof(double) * t64.size());
    if (e == cudaSuccess && !c->d_dense32) e = cudaMalloc(&c->d_dense32, sizeof(float) * t32.size());
    if (e != cudaSuccess) return fail(HLBL_ENOMEM, "hlbl_ctx_set_qed_kernel: %s", cudaGetErrorString(e));
    // ordered on the context's stream after every launch that reads the old table
    e = cudaMemcpyAsync(c->d_dense64, t64.data(), sizeof(double) * t64.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->d_dense32, t32.data(), sizeof(float) * t32.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "hlbl_ctx_set_qed_kernel: table upload");
  }
  c->qed_kind = kind;
  return HLBL_OK;
}

int hlbl_ctx_set_qed(hlbl_ctx* c, int mode, hlbl_surrogate* s, double r0) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_qed: null context");
  if (mode == HLBL_QED_SURROGATE && c->qed_kind != kQedStandInClosed)
    return fail(HLBL_ESTATE, "hlbl_ctx_set_qed: the learned weight replaces the stand-in's closed form only");
  if (mode == HLBL_QED_EXACT) {
    c->qed_mode = mode;
    c->sur = nullptr;
    return HLBL_OK;
  }
  if (mode != HLBL_QED_SURROGATE || !s) return fail(HLBL_EINVAL, "hlbl_ctx_set_qed: bad mode or null surrogate");
  if (!c->d_fallback) {
    cudaError_t e = cudaMalloc(&c->d_fallback, sizeof(unsigned long long));
    if (e != cudaSuccess) return fail(HLBL_ENOMEM, "hlbl_ctx_set_qed: %s", cudaGetErrorString(e));
  }
  cudaError_t e = cudaMemsetAsync(c->d_fallback, 0, sizeof(unsigned long long), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_ctx_set_qed");
  c->qed_mode = mode;
  c->sur = s;
  c->sur_r0 = r0 < 0 ? sur::surrogate_r0(s) : r0;
  return HLBL_OK;
}

int hlbl_ctx_qed_fallbacks(hlbl_ctx* c, unsigned long long* n) {
  if (!c || !n) return fail(HLBL_EINVAL, "hlbl_ctx_qed_fallbacks: null argument");
  *n = 0;
  if (!c->d_fallback) return HLBL_OK;
  cudaError_t e = cudaMemcpyAsync(n, c->d_fallback, sizeof *n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? HLBL_OK : cuda_fail(e, "hlbl_ctx_qed_fallbacks");
}

int hlbl_ctx_set_profiling(hlbl_ctx* c, int on) {
  if (!c) return fail(HLBL_EINVAL, "hlbl_ctx_set_profiling: null context");
  if (on && !c->ev[0][0]) {
    for (auto& pe : c->ev)
      for (auto& e : pe) {
        cudaError_t er = cudaEventCreate(&e);
        if (er != cudaSuccess) return cuda_fail(er, "cudaEventCreate");
      }
  }
  c->profiling = on != 0;
  c->prof_ms[0] = c->prof_ms[1] = 0;
  c->prof_n[0] = c->prof_n[1] = 0;
  c->prof_pending[0] = c->prof_pending[1] = 0;
  return HLBL_OK;
}

int hlbl_ctx_kernel_times(hlbl_ctx* c, double ms[2], long long n[2]) {
  if (!c || !ms || !n) return fail(HLBL_EINVAL, "hlbl_ctx_kernel_times: null argument");
  prof_collect(c, 0);
  prof_collect(c, 1);
  for (int p = 0; p < 2; ++p) { ms[p] = c->prof_ms[p]; n[p] = c->prof_n[p]; }
  return HLBL_OK;
}

int hlbl_fill_random_block(hlbl_ctx* c, double* d_out, uint64_t seed) {
  if (!c || !d_out) return fail(HLBL_EINVAL, "hlbl_fill_random_block: null argument");
  fill_uniform_kernel<<<c->nsm * 8, 256, 0, c->stream>>>(d_out, c->geo, seed);
  return check_launch("hlbl_fill_random_block launch");
}

int hlbl_fill_gaussian_block(hlbl_ctx* c, double* d_out, uint64_t seed) {
  if (!c || !d_out) return fail(HLBL_EINVAL, "hlbl_fill_gaussian_block: null argument");
  if (!aligned16(d_out)) return fail(HLBL_EINVAL, "hlbl_fill_gaussian_block: block must be 16-byte aligned");
  fill_gaussian_kernel<<<c->nsm * 8, 256, 0, c->stream>>>(d_out, c->geo, seed);
  return check_launch("hlbl_fill_gaussian_block launch");
}

}  // extern "C"
