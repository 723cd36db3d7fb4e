// ref_gpu_capi.cpp -- TEST INFRASTRUCTURE. A C entry layer over the GPU build
// of the reference's own sources (oracle/ref_gpu/Makefile): its Contractor
// (src/contract.cpp) driving its vendored kernels (kernels/cuda_lattice.cu,
// kernels/hlbl_kernels/kernels.cu) on the GPU, single rank. The tests check the
// library against it and bench.py times it as the same-box GPU baseline.
// Never shipped.
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "hlbl/contract.hpp"

namespace {
thread_local std::string g_err;

struct RefGpu {
  std::unique_ptr<hlbl::Lattice> lat;
  std::unique_ptr<hlbl::Contractor> con;
  QED_kernel_temps kq{};
  double* d_dense = nullptr;
};

hlbl::Vec4 v4(const int v[4]) { return hlbl::Vec4{v[0], v[1], v[2], v[3]}; }

int failed(const std::exception& e) {
  g_err = e.what();
  return 1;
}
}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err.c_str(); }

// One rank holding the whole lattice `local`; dense != 0: the dense test
// weight with its table seeded by `seed`, else the stand-in.
int refgpu_create(void** out, const int local[4], int dense, unsigned long long seed) {
  try {
    auto* r = new RefGpu();
    initialise(&r->kq);
    if (dense) {
      std::vector<double> t((std::size_t)HLBL_QED_DENSE_NB * HLBL_QED_NK);
      hlbl_qed_dense_init(t.data(), seed);
      hlbl::check_cuda(cudaMalloc(&r->d_dense, t.size() * sizeof(double)), "dense table");
      hlbl::check_cuda(cudaMemcpy(r->d_dense, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice),
                       "dense table");
      r->kq.dense = r->d_dense;
    }
    r->lat = std::make_unique<hlbl::Lattice>(MPI_COMM_WORLD, hlbl::Vec4{1, 1, 1, 1}, v4(local));
    r->con = std::make_unique<hlbl::Contractor>(*r->lat, r->kq);
    *out = r;
    return 0;
  } catch (const std::exception& e) {
    return failed(e);
  }
}

void refgpu_destroy(void* h) {
  auto* r = static_cast<RefGpu*>(h);
  if (!r) return;
  r->con.reset();
  r->lat.reset();
  if (r->d_dense) cudaFree(r->d_dense);
  delete r;
}

// Contractor::kernel_sum (src/contract.cpp:104-114) on device blocks.
int refgpu_kernel_sum(void* h, const double* d_src, const double* d_y, const int gsx[4], const int yv[4],
                      double xunit, double out[2]) {
  try {
    auto r = static_cast<RefGpu*>(h)->con->kernel_sum(d_src, d_y, v4(gsx), v4(yv), xunit);
    out[0] = r[0];
    out[1] = r[1];
    return 0;
  } catch (const std::exception& e) {
    return failed(e);
  }
}

// Contractor::pieces_2p2 (src/contract.cpp:116-156): p1 [4][4][4][Lmax],
// p234 [n_y][5][64].
int refgpu_pieces_2p2(void* h, const double* d_fwd, const int gsw[4], const int* targets, int n_y,
                      double xunit, double* p1, double* p234) {
  try {
    std::vector<hlbl::Vec4> tg;
    for (int t = 0; t < n_y; ++t) tg.push_back(v4(targets + 4 * t));
    auto pc = static_cast<RefGpu*>(h)->con->pieces_2p2(d_fwd, v4(gsw), tg, xunit);
    std::memcpy(p1, pc.p1.data(), pc.p1.size() * sizeof(double));
    std::memcpy(p234, pc.p234.data(), pc.p234.size() * sizeof(double));
    return 0;
  } catch (const std::exception& e) {
    return failed(e);
  }
}

// Contractor::reserve_kernel_memory (src/contract.cpp:158-197).
int refgpu_reserve_kernel_memory(void* h, int with_2p2, std::size_t* bytes) {
  try {
    *bytes = static_cast<RefGpu*>(h)->con->reserve_kernel_memory(with_2p2 != 0);
    return 0;
  } catch (const std::exception& e) {
    return failed(e);
  }
}

}  // extern "C"
