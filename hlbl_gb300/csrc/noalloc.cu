// noalloc.cu -- pass 1 (hlbl_cu_dzu_dzsu) for callers that cannot allocate
// device memory at the time they contract.
//
// The reference's production runs contract next to a solver (tmLQCD/QUDA)
// that has already taken nearly all device memory into its own pool, and
// the preflight measures free memory around the kernels
// (Contractor::reserve_kernel_memory). Such a caller cannot create a
// context, which allocates its work buffers. This entry point needs none:
// the per-thread-block partial sums of pass 1 and one error word live in
// fixed arrays in this library's device image, which every GPU that loads
// the library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "contract_kernels.cuh"
#include "hlbl_gb300.h"
#include "hlbl_internal.h"

namespace {

using Kernel = hg::P1NoAllocTraits;

// One 2,880-double slot of partial sums per thread block, for at most
// HLBL_NOALLOC_MAX_BLOCKS blocks: 512 x 2880 x 8 B = 11.8 MB. Pass 1 strides
// over the lattice's tiles, so its grid is capped at that many blocks and
// any lattice fits.
static __device__ __align__(256) double g_partials[HLBL_NOALLOC_MAX_BLOCKS * hg::kDzLen];
// Set by a pass-1 block that gave up a bounded wait for a staged tile (it
// then skips writing its slot); cleared at the start of every call.
static __device__ __align__(256) int g_err;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_partials_addr[kMaxDevices] = {};  // device address of g_partials, per device
int* g_err_addr[kMaxDevices] = {};          // device address of g_err, per device
int g_resident[kMaxDevices] = {};           // resident pass-1 blocks on that device

// Adds the fixed-order, compensated sum of the partials into the caller's
// dzu[1728] and dzsu[1152]; allocates nothing. If a pass-1 block gave up
// (its slot holds an earlier call's sums), every output becomes NaN, so the
// failure cannot pass as a result.
__global__ void noalloc_reduce_kernel(const double* __restrict__ partials, int nblocks,
                                      const int* __restrict__ err, double* __restrict__ dzu,
                                      double* __restrict__ dzsu) {
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hg::kDzLen) return;
  hg::Neu s;
  for (int b = 0; b < nblocks; ++b) s.add(partials[(size_t)b * hg::kDzLen + i]);
  double const v = *err ? __longlong_as_double(0x7ff8000000000000LL) : s.get();
  if (i < hg::kDzuLen) dzu[i] += v;
  else dzsu[i - hg::kDzuLen] += v;
}

// Once per device, with that device current: the device addresses of the
// scratch array and the error word (host code may not use the symbols
// themselves) and the number of resident pass-1 blocks.
int setup(int dev, double** addr, int** err, int* resident) {
  if (dev < 0 || dev >= kMaxDevices) return hg::fail(HLBL_EINVAL, "noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    void* q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: cudaGetSymbolAddress(partials)");
    e = cudaGetSymbolAddress(&q, g_err);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: cudaGetSymbolAddress(error word)");
    e = cudaFuncSetAttribute(hg::p1_kernel<double, 1, Kernel::kTS>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Kernel::kSmem);
    // the same carveout as the context's pass 1, so the occupancy is the same
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(hg::p1_kernel<double, 1, Kernel::kTS>,
                               cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: smem attribute");
    int nb = 0, nsm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, hg::p1_kernel<double, 1, Kernel::kTS>,
                                                      Kernel::kThreads, Kernel::kSmem);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: occupancy");
    if (nb < 1) return hg::fail(HLBL_ECUDA, "noalloc: pass 1 cannot be resident (smem %zu)", Kernel::kSmem);
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: SM count");
    g_resident[dev] = nb * nsm;
    g_err_addr[dev] = static_cast<int*>(q);
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *addr = g_partials_addr[dev];
  *err = g_err_addr[dev];
  *resident = g_resident[dev];
  return HLBL_OK;
}

}  // namespace

extern "C" int hlbl_cu_dzu_dzsu_noalloc(double* d_dzu, double* d_dzsu, const double* fwd_src,
                                        const double* fwd_y, int iflavor, const int pc[4],
                                        const int gsx[4], const int global_geom[4],
                                        const int local_geom[4], void* stream) {
  if (!d_dzu || !d_dzsu || !fwd_src || !fwd_y || !pc || !gsx || !global_geom || !local_geom)
    return hg::fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu_noalloc: null argument");
  if (iflavor != 0 && iflavor != 1)
    return hg::fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu_noalloc: iflavor must be 0 or 1");
  if ((reinterpret_cast<uintptr_t>(fwd_src) | reinterpret_cast<uintptr_t>(fwd_y)) & 15u)
    return hg::fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu_noalloc: blocks must be 16-byte aligned");
  hg::Geometry geo{};
  long long V = 1;
  for (int r = 0; r < 4; ++r) {
    if (local_geom[r] < 1 || global_geom[r] < 1 || pc[r] < 0 ||
        (long long)(pc[r] + 1) * local_geom[r] > global_geom[r])
      return hg::fail(HLBL_EINVAL, "hlbl_cu_dzu_dzsu_noalloc: bad geometry in direction %d", r);
    geo.local[r] = local_geom[r];
    geo.global[r] = global_geom[r];
    geo.pc[r] = pc[r];
    V *= local_geom[r];
  }
  geo.V = V;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hg::cuda_fail(e, "hlbl_cu_dzu_dzsu_noalloc: cudaGetDevice");
  double* partials = nullptr;
  int* err = nullptr;
  int resident = 0;
  if (int rc = setup(dev, &partials, &err, &resident)) return rc;
  // pass 1 strides over the tiles: any grid of at least one block gives the
  // same sums, so the grid is capped at the scratch's slots
  long long const tiles = (V + Kernel::kTS - 1) / Kernel::kTS;
  long long nb = tiles < resident ? tiles : resident;
  if (nb > HLBL_NOALLOC_MAX_BLOCKS) nb = HLBL_NOALLOC_MAX_BLOCKS;
  int const nblocks = (int)nb;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every block that finishes writes its whole slot, so the partials need no
  // clearing; the error word does
  e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e != cudaSuccess) return hg::cuda_fail(e, "hlbl_cu_dzu_dzsu_noalloc: error word clear");
  hg::PairBatch b{};
  b.n = 1;
  b.p[0].src = fwd_src;
  for (int r = 0; r < 4; ++r) b.p[0].gsx[r] = gsx[r];
  hg::p1_kernel<double, 1, Kernel::kTS><<<dim3(nblocks, 1), Kernel::kThreads, Kernel::kSmem, st>>>(
      fwd_y, b, geo, iflavor, partials, err, nullptr);
  noalloc_reduce_kernel<<<(hg::kDzLen + 255) / 256, 256, 0, st>>>(partials, nblocks, err, d_dzu, d_dzsu);
  e = cudaGetLastError();
  if (e != cudaSuccess) return hg::cuda_fail(e, "hlbl_cu_dzu_dzsu_noalloc launch");
  return HLBL_OK;
}
