// noalloc.cu -- pass 1 (hlbl_cu_dzu_dzsu) for callers that cannot allocate
// device memory at the time they contract.
//
// The reference's production runs contract next to a solver (tmLQCD/QUDA)
// that has already taken nearly all device memory into its own pool, and
// the preflight measures free memory around the kernels
// (Contractor::reserve_kernel_memory). Such a caller cannot create a
// context, which allocates its work buffers. This entry point needs none:
// the per-thread-block partial sums of pass 1 live in a fixed array in this
// library's device image, which every GPU that loads the library holds
// until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "contract_kernels.cuh"
#include "hlbl_gb300.h"
#include "hlbl_internal.h"

namespace {

using Kernel = hg::P1NoAllocTraits;

// One 2,880-double slot of partial sums per thread block, for at most
// HLBL_NOALLOC_MAX_BLOCKS blocks: 512 x 2880 x 8 B = 11.8 MB. A call whose
// pass 1 would run more resident blocks than that is rejected.
static __device__ __align__(256) double g_partials[HLBL_NOALLOC_MAX_BLOCKS * hg::kDzLen];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_partials_addr[kMaxDevices] = {};  // device address of g_partials, per device
int g_resident[kMaxDevices] = {};           // resident pass-1 blocks on that device

// Adds the fixed-order, compensated sum of the partials into the caller's
// dzu[1728] and dzsu[1152]; allocates nothing.
__global__ void noalloc_reduce_kernel(const double* __restrict__ partials, int nblocks,
                                      double* __restrict__ dzu, double* __restrict__ dzsu) {
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hg::kDzLen) return;
  hg::Neu s;
  for (int b = 0; b < nblocks; ++b) s.add(partials[(size_t)b * hg::kDzLen + i]);
  double const v = s.get();
  if (i < hg::kDzuLen) dzu[i] += v;
  else dzsu[i - hg::kDzuLen] += v;
}

// Once per device, with that device current: the device address of the
// scratch array (host code may not use the symbol itself) and the number of
// resident pass-1 blocks.
int setup(int dev, double** addr, int* resident) {
  if (dev < 0 || dev >= kMaxDevices) return hg::fail(HLBL_EINVAL, "noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: cudaGetSymbolAddress");
    e = cudaFuncSetAttribute(hg::p1_kernel<double, 1, Kernel::kTS>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Kernel::kSmem);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: smem attribute");
    int nb = 0, nsm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, hg::p1_kernel<double, 1, Kernel::kTS>,
                                                      Kernel::kThreads, Kernel::kSmem);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: occupancy");
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return hg::cuda_fail(e, "noalloc: SM count");
    g_resident[dev] = nb * nsm;
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *addr = g_partials_addr[dev];
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
  int resident = 0;
  if (int rc = setup(dev, &partials, &resident)) return rc;
  long long const tiles = (V + Kernel::kTS - 1) / Kernel::kTS;
  int const nblocks = (int)(tiles < resident ? tiles : resident);
  if (nblocks > HLBL_NOALLOC_MAX_BLOCKS)
    return hg::fail(HLBL_EINVAL,
                    "hlbl_cu_dzu_dzsu_noalloc: pass 1 runs %d thread blocks on this device; its "
                    "fixed scratch holds partial sums for at most %d",
                    nblocks, HLBL_NOALLOC_MAX_BLOCKS);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every block writes its whole slot, so nothing has to be cleared first
  hg::PairBatch b{};
  b.n = 1;
  b.p[0].src = fwd_src;
  for (int r = 0; r < 4; ++r) b.p[0].gsx[r] = gsx[r];
  hg::p1_kernel<double, 1, Kernel::kTS><<<dim3(nblocks, 1), Kernel::kThreads, Kernel::kSmem, st>>>(
      fwd_y, b, geo, iflavor, partials, nullptr, nullptr);
  noalloc_reduce_kernel<<<(hg::kDzLen + 255) / 256, 256, 0, st>>>(partials, nblocks, d_dzu, d_dzsu);
  e = cudaGetLastError();
  if (e != cudaSuccess) return hg::cuda_fail(e, "hlbl_cu_dzu_dzsu_noalloc launch");
  return HLBL_OK;
}
