// cuda_lattice_gb300.cpp -- the reference's vendored launchers cu_dzu_dzsu and
// cu_4pt_contraction (kernels/cuda_lattice.h:49-57, kernels/cuda_lattice.cu:792-839)
// over libhlbl_gb300.so, for C++ callers that link this file instead of
// kernels/cuda_lattice.cu. The reference's src/contract.cpp, src/driver.cpp
// and everything above them compile unchanged against the reference's own
// headers (cuda_lattice.h, KQED.h, mpi.h) and link with this file and the
// library.
//
// Same arguments and meaning as the vendored launchers: results are ADDED into
// caller-zeroed device buffers, FP64 products and sums, asynchronous. The
// launches run on a library context per (device, lattice, rank position),
// made on first use and kept for the process; its stream is a blocking
// stream, so the caller's synchronous copies on the legacy default stream
// (contract.cpp:47-48, :98) wait for them. The QED kernel is the library's
// (the kqed_t argument is not read). Errors throw std::runtime_error with
// the library's message (the vendored launchers report only through
// cudaGetLastError, which contract.cpp checks after each launch).
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>

#include "cuda_lattice.h"
#include "hlbl_gb300.h"
#include "hlbl_gb300_dropin.h"

namespace {

using Key = std::tuple<int, int, int, int, int, int, int, int, int, int, int, int, int>;

std::mutex g_mu;
std::map<Key, hlbl_ctx*> g_ctx;

void check(int rc, const char* what) {
  if (rc != HLBL_OK) throw std::runtime_error(std::string(what) + ": " + hlbl_last_error());
}

}  // namespace

hlbl_ctx* hlbl_dropin_context(const int global[4], const int local[4], const int pc[4]) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) throw std::runtime_error("hlbl dropin: cudaGetDevice failed");
  Key const key{dev, global[0], global[1], global[2], global[3], local[0], local[1], local[2], local[3],
                pc[0], pc[1], pc[2], pc[3]};
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_ctx.find(key);
  if (it != g_ctx.end()) return it->second;
  hlbl_ctx* c = nullptr;
  // LLambda with Lambda = 0.4 (KQED_LX, cuda_lattice.cu:266-275)
  check(hlbl_ctx_create(&c, global, local, pc, 0.4, dev), "hlbl_ctx_create");
  g_ctx[key] = c;
  return c;
}

void cu_dzu_dzsu(double* d_dzu, double* d_dzsu, const double* fwd_src, const double* fwd_y, int iflavor,
                 Coord proc_coords, Coord gsx, Geom global_geom, Geom local_geom) {
  int const pc[4] = {proc_coords.t, proc_coords.x, proc_coords.y, proc_coords.z};
  int const s[4] = {gsx.t, gsx.x, gsx.y, gsx.z};
  int const g[4] = {global_geom.T, global_geom.LX, global_geom.LY, global_geom.LZ};
  int const l[4] = {local_geom.T, local_geom.LX, local_geom.LY, local_geom.LZ};
  check(hlbl_cu_dzu_dzsu(hlbl_dropin_context(g, l, pc), d_dzu, d_dzsu, fwd_src, fwd_y, iflavor, pc, s, g, l),
        "cu_dzu_dzsu");
}

void cu_4pt_contraction(double* d_kernel_sum, const double* d_g_dzu, const double* d_g_dzsu,
                        const double* fwd_src, const double* fwd_y, int iflavor, Coord proc_coords, Coord gsx,
                        Pair xunit, Coord yv, QED_kernel_temps /*kqed_t*/, Geom global_geom, Geom local_geom) {
  int const pc[4] = {proc_coords.t, proc_coords.x, proc_coords.y, proc_coords.z};
  int const s[4] = {gsx.t, gsx.x, gsx.y, gsx.z};
  int const y[4] = {yv.t, yv.x, yv.y, yv.z};
  int const g[4] = {global_geom.T, global_geom.LX, global_geom.LY, global_geom.LZ};
  int const l[4] = {local_geom.T, local_geom.LX, local_geom.LY, local_geom.LZ};
  check(hlbl_cu_4pt_contraction(hlbl_dropin_context(g, l, pc), d_kernel_sum, d_g_dzu, d_g_dzsu, fwd_src, fwd_y,
                                iflavor, pc, s, xunit.a, y, g, l),
        "cu_4pt_contraction");
}
