// kernels_2p2_gb300.cpp -- the reference's compute_2p2_gpu
// (kernels/hlbl_kernels/kernels.cuh:10-13, kernels.cu:753-870) over
// libhlbl_gb300.so, for C++ callers that link this file instead of
// kernels/hlbl_kernels/kernels.cu; src/contract.cpp (Contractor::pieces_2p2,
// reserve_kernel_memory) compiles and links unchanged.
//
// Same arguments and meaning: P1 [4][4][4][Lmax] and P234 [5][n_y][64] host
// arrays, overwritten with the sums over all ranks of g_cart_grid (the
// reference's in-place MPI_Iallreduce, kernels.cu:824-860, done here as
// MPI_Allreduce). gsw, xunit and g_proc_coords may be device pointers, as
// Contractor passes them (contract.cpp:134-143), or host pointers. FP64
// products and sums; blocking. The library's QED kernel weights (kqed_t is
// not read).
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "hlbl_gb300.h"
#include "hlbl_gb300_dropin.h"
#include "kernels.cuh"

namespace {

// a small argument array from device or host memory (unified addressing)
template <typename T>
void fetch(T* dst, const T* src, int n) {
  if (cudaMemcpy(dst, src, sizeof(T) * n, cudaMemcpyDefault) != cudaSuccess)
    throw std::runtime_error("compute_2p2_gpu: cannot read an argument array");
}

}  // namespace

__host__ void compute_2p2_gpu(double* fwd_y, double* P1, double* P234, int const iflavor, int const gsw[4],
                              const int* gycoords, int const n_y, const double xunit[2], QED_kernel_temps /*kqed_t*/,
                              unsigned const VOLUME, int const g_proc_coords[4], MPI_Comm g_cart_grid,
                              unsigned const T, unsigned const LX, unsigned const LY, unsigned const LZ,
                              unsigned const T_global, unsigned const LX_global, unsigned const LY_global,
                              unsigned const LZ_global) {
  int w[4], pc[4];
  double xu[2];
  fetch(w, gsw, 4);
  fetch(pc, g_proc_coords, 4);
  fetch(xu, xunit, 2);
  int const g[4] = {(int)T_global, (int)LX_global, (int)LY_global, (int)LZ_global};
  int const l[4] = {(int)T, (int)LX, (int)LY, (int)LZ};
  if ((unsigned long long)l[0] * l[1] * l[2] * l[3] != VOLUME)
    throw std::runtime_error("compute_2p2_gpu: VOLUME is not the product of the local extents");
  hlbl_ctx* c = hlbl_dropin_context(g, l, pc);
  int const rc = hlbl_compute_2p2(c, fwd_y, P1, P234, iflavor, w, gycoords, n_y, xu[0], HLBL_FP64);
  if (rc != HLBL_OK) throw std::runtime_error(std::string("compute_2p2_gpu: ") + hlbl_last_error());
  int lmax = g[0];
  for (int r = 1; r < 4; ++r) lmax = g[r] > lmax ? g[r] : lmax;
  MPI_Allreduce(MPI_IN_PLACE, P1, 64 * lmax, MPI_DOUBLE, MPI_SUM, g_cart_grid);
  MPI_Allreduce(MPI_IN_PLACE, P234, 5 * 64 * n_y, MPI_DOUBLE, MPI_SUM, g_cart_grid);
}
