// capi.cu -- the C ABI of libhlbl_gb300.so: the contraction context, its
// work buffers and stream, kernel launch plumbing, and the entry points
// declared in include/hlbl_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "contract_kernels.cuh"
#include "hlbl_gb300.h"
#include "hlbl_gb300_rng.h"
#include "hlbl_internal.h"

namespace {

thread_local std::string g_last_error;

}  // namespace

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

// ---- launch plumbing -------------------------------------------------------
template <typename T, int NF, int TS>
struct P1Launch {
  static constexpr int threads = NF * 144;
  static constexpr size_t smem = p1_smem_bytes<T, NF, TS>();
  static int init(int nsm, int& grid) {
    cudaError_t e = cudaFuncSetAttribute(p1_kernel<T, NF, TS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "p1 smem attribute");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, p1_kernel<T, NF, TS>, threads, smem);
    if (e != cudaSuccess) return cuda_fail(e, "p1 occupancy");
    if (nb < 1) return fail(HLBL_ECUDA, "p1 kernel cannot be resident (smem %zu)", smem);
    grid = nb * nsm;
    return HLBL_OK;
  }
  static void launch(int grid, cudaStream_t st, const double* src, const double* y,
                     const Geometry& geo, int4 gsx, int f0, double* partials) {
    p1_kernel<T, NF, TS><<<grid, threads, smem, st>>>(src, y, geo, gsx, f0, partials);
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
  static void launch(int grid, cudaStream_t st, const double* src, const double* y,
                     const Geometry& geo, const P2Args& a, const T* bt, double* partials) {
    p2_kernel<T, NF, TS><<<grid, threads, smem, st>>>(src, y, geo, a, bt, partials);
  }
  static long long tiles(long long V) { return (V + TS - 1) / TS; }
};

// tile sizes per precision
using P1D2 = P1Launch<double, 2, 16>;
using P1D1 = P1Launch<double, 1, 16>;
using P1F2 = P1Launch<float, 2, 32>;
using P1F1 = P1Launch<float, 1, 32>;
using P2D2 = P2Launch<double, 2, 4>;
using P2D1 = P2Launch<double, 1, 4>;
using P2F2 = P2Launch<float, 2, 8>;
using P2F1 = P2Launch<float, 1, 8>;

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
  int grid_p1d2 = 0, grid_p1d1 = 0, grid_p1f2 = 0, grid_p1f1 = 0;
  int grid_p2d2 = 0, grid_p2d1 = 0, grid_p2f2 = 0, grid_p2f1 = 0;
  int max_grid = 0;
  double* d_part1 = nullptr;  // [max_grid][2][2880]
  double* d_part2 = nullptr;  // [max_grid][2]
  double* d_dz = nullptr;     // [2][2880]
  double* d_g = nullptr;      // [2][11520]
  void* d_bt = nullptr;       // [2][288*160] of double (float uses half of it)
  double* d_out = nullptr;    // [2]
  double* h_out = nullptr;    // pinned [2]
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
  if (!c->profiling) return;
  prof_collect(c, pass);
  cudaEventRecord(c->ev[pass][0], c->stream);
}
void prof_end(hlbl_ctx* c, int pass) {
  if (!c->profiling) return;
  cudaEventRecord(c->ev[pass][1], c->stream);
  c->prof_pending[pass] = 1;
}

// Pass 1 + reduction + gamma insertion + Bt for flavours [f0, f0+nf).
// g_dzu/g_dzsu of flavour fl land at d_g + fl*kGLen (+kGDzuLen).
int run_pass1(hlbl_ctx* c, const Geometry& geo, const double* src, const double* y,
              const int gsx[4], int f0, int nf, int precision, double* add_dzu,
              double* add_dzsu, bool build_bt) {
  int4 const g4 = make_int4(gsx[0], gsx[1], gsx[2], gsx[3]);
  int grid;
  prof_begin(c, 0);
  if (precision == HLBL_FP64) {
    if (nf == 2) { grid = (int)std::min<long long>(c->grid_p1d2, P1D2::tiles(geo.V)); P1D2::launch(grid, c->stream, src, y, geo, g4, f0, c->d_part1); }
    else { grid = (int)std::min<long long>(c->grid_p1d1, P1D1::tiles(geo.V)); P1D1::launch(grid, c->stream, src, y, geo, g4, f0, c->d_part1); }
  } else {
    if (nf == 2) { grid = (int)std::min<long long>(c->grid_p1f2, P1F2::tiles(geo.V)); P1F2::launch(grid, c->stream, src, y, geo, g4, f0, c->d_part1); }
    else { grid = (int)std::min<long long>(c->grid_p1f1, P1F1::tiles(geo.V)); P1F1::launch(grid, c->stream, src, y, geo, g4, f0, c->d_part1); }
  }
  prof_end(c, 0);
  p1_reduce_kernel<<<dim3((kDzLen + 255) / 256, nf), 256, 0, c->stream>>>(c->d_part1, grid, nf, c->d_dz,
                                                                          add_dzu, add_dzsu);
  if (!build_bt) return HLBL_OK;
  g_build_kernel<<<dim3((kGLen / 2 + 255) / 256, nf), 256, 0, c->stream>>>(c->d_dz, nf, c->d_g);
  if (precision == HLBL_FP64)
    bt_build_kernel<double><<<dim3((kBtK * kBtN + 255) / 256, nf), 256, 0, c->stream>>>(
        c->d_g, c->d_g + kGDzuLen, kGLen, nf, static_cast<double*>(c->d_bt));
  else
    bt_build_kernel<float><<<dim3((kBtK * kBtN + 255) / 256, nf), 256, 0, c->stream>>>(
        c->d_g, c->d_g + kGDzuLen, kGLen, nf, static_cast<float*>(c->d_bt));
  return HLBL_OK;
}

// Pass 2 for flavours [f0, f0+nf) with Bt already built; reduces into
// out[0..nf) (added if add).
int run_pass2(hlbl_ctx* c, const Geometry& geo, const double* src, const double* y,
              const int gsx[4], const int yv[4], double xunit, int f0, int nf, int precision,
              double* out, int add) {
  P2Args a{};
  for (int r = 0; r < 4; ++r) { a.gsx[r] = gsx[r]; a.yv[r] = yv[r]; }
  a.xunit = xunit;
  a.f0 = f0;
  a.qp = c->qp;
  int grid;
  prof_begin(c, 1);
  if (precision == HLBL_FP64) {
    const double* bt = static_cast<const double*>(c->d_bt);
    if (nf == 2) { grid = (int)std::min<long long>(c->grid_p2d2, P2D2::tiles(geo.V)); P2D2::launch(grid, c->stream, src, y, geo, a, bt, c->d_part2); }
    else { grid = (int)std::min<long long>(c->grid_p2d1, P2D1::tiles(geo.V)); P2D1::launch(grid, c->stream, src, y, geo, a, bt, c->d_part2); }
  } else {
    const float* bt = static_cast<const float*>(c->d_bt);
    if (nf == 2) { grid = (int)std::min<long long>(c->grid_p2f2, P2F2::tiles(geo.V)); P2F2::launch(grid, c->stream, src, y, geo, a, bt, c->d_part2); }
    else { grid = (int)std::min<long long>(c->grid_p2f1, P2F1::tiles(geo.V)); P2F1::launch(grid, c->stream, src, y, geo, a, bt, c->d_part2); }
  }
  prof_end(c, 1);
  p2_reduce_kernel<<<1, 32, 0, c->stream>>>(c->d_part2, grid, nf, out, add);
  return HLBL_OK;
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
  auto bail = [&](int rc) { hlbl_ctx_destroy(c); return rc; };
  e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return bail(cuda_fail(e, "SM count"));
  int rc;
  if ((rc = P1D2::init(c->nsm, c->grid_p1d2)) || (rc = P1D1::init(c->nsm, c->grid_p1d1)) ||
      (rc = P1F2::init(c->nsm, c->grid_p1f2)) || (rc = P1F1::init(c->nsm, c->grid_p1f1)) ||
      (rc = P2D2::init(c->nsm, c->grid_p2d2)) || (rc = P2D1::init(c->nsm, c->grid_p2d1)) ||
      (rc = P2F2::init(c->nsm, c->grid_p2f2)) || (rc = P2F1::init(c->nsm, c->grid_p2f1)))
    return bail(rc);
  c->max_grid = std::max({c->grid_p1d2, c->grid_p1d1, c->grid_p1f2, c->grid_p1f1, c->grid_p2d2,
                          c->grid_p2d1, c->grid_p2f2, c->grid_p2f1});
  e = cudaStreamCreate(&c->own_stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
  c->stream = c->own_stream;
  struct { void** p; size_t n; } bufs[] = {
      {(void**)&c->d_part1, sizeof(double) * (size_t)c->max_grid * 2 * kDzLen},
      {(void**)&c->d_part2, sizeof(double) * (size_t)c->max_grid * 2},
      {(void**)&c->d_dz, sizeof(double) * 2 * kDzLen},
      {(void**)&c->d_g, sizeof(double) * 2 * kGLen},
      {(void**)&c->d_bt, sizeof(double) * 2 * kBtK * kBtN},
      {(void**)&c->d_out, sizeof(double) * 2}};
  for (auto& b : bufs) {
    e = cudaMalloc(b.p, b.n);
    if (e != cudaSuccess) return bail(fail(HLBL_ENOMEM, "cudaMalloc %zu bytes: %s", b.n, cudaGetErrorString(e)));
  }
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
  cudaFree(c->d_out);
  if (c->h_out) cudaFreeHost(c->h_out);
  for (auto& pe : c->ev)
    for (auto& e : pe)
      if (e) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
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
  if (int rc = run_pass1(c, c->geo, src, y, gsx, 0, 2, precision, nullptr, nullptr, true)) return rc;
  if (int rc = run_pass2(c, c->geo, src, y, gsx, yv, xunit, 0, 2, precision, d_out, 0)) return rc;
  return check_launch("hlbl_kernel_sum launch");
}

int hlbl_kernel_sum(hlbl_ctx* c, const double* src, const double* y, const int gsx[4],
                    const int yv[4], double xunit, int precision, double out[2]) {
  if (!out) return fail(HLBL_EINVAL, "hlbl_kernel_sum: null out");
  if (int rc = hlbl_kernel_sum_async(c, src, y, gsx, yv, xunit, precision, c ? c->d_out : nullptr)) return rc;
  cudaError_t e = cudaMemcpyAsync(c->h_out, c->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "result copy");
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_kernel_sum");
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
  if (int rc = run_pass1(c, geo, src, y, gsx, iflavor, 1, HLBL_FP64, d_dzu, d_dzsu, false)) return rc;
  return check_launch("hlbl_cu_dzu_dzsu launch");
}

int hlbl_insert_gammas(hlbl_ctx* c, const double* d_dzu, const double* d_dzsu, double* d_g_dzu,
                       double* d_g_dzsu) {
  if (!c || !d_dzu || !d_dzsu || !d_g_dzu || !d_g_dzsu) return fail(HLBL_EINVAL, "hlbl_insert_gammas: null argument");
  cudaError_t e = cudaMemcpyAsync(c->d_dz, d_dzu, kDzuLen * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_dz + kDzuLen, d_dzsu, (kDzLen - kDzuLen) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hlbl_insert_gammas copy");
  g_build_kernel<<<dim3((kGLen / 2 + 255) / 256, 1), 256, 0, c->stream>>>(c->d_dz, 1, c->d_g);
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
  bt_build_kernel<double><<<dim3((kBtK * kBtN + 255) / 256, 1), 256, 0, c->stream>>>(
      d_g_dzu, d_g_dzsu, 0, 1, static_cast<double*>(c->d_bt));
  if (int rc = run_pass2(c, geo, src, y, gsx, yv, xunit, iflavor, 1, HLBL_FP64, d_ks, 1)) return rc;
  return check_launch("hlbl_cu_4pt_contraction launch");
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
        run_pass1(c, geo, blk, blk, zero, 0, nf, prec, nullptr, nullptr, true);
        run_pass2(c, geo, blk, blk, zero, one, 1.0, 0, nf, prec, c->d_out, 0);
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
