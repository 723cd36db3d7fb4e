// ref_capi.cpp -- TEST INFRASTRUCTURE. A C entry layer over the reference's
// own sources (kernels/cuda_lattice.cu, kernels/hlbl_kernels/kernels.cu,
// src/contract.cpp, src/provider.cpp, src/gamma.cpp, src/geometry.cpp,
// src/schedule.cpp), compiled as a host
// emulation with the shims in ./shim. It lets the fixture script run the
// reference's code on small lattices to pin the oracle. Never shipped.
#include <algorithm>
#include <cstdint>
#include <string>
#include <stdexcept>
#include <vector>

#include "hlbl/contract.hpp"
#include "hlbl/gamma.hpp"
#include "hlbl/provider.hpp"
#include "hlbl/schedule.hpp"
#include "hlbl_kernels/kernels.cuh"

// KQED entry points, served by the stand-in weight or, after
// ref_set_qed_dense, by the dense test weight (include/hlbl_gb300_qed.h)
static std::vector<double> g_dense;  // empty: the stand-in

extern "C" int initialise(struct QED_kernel_temps* t) {
  hlbl_qed_params_init(&t->p, 0.4);
  return 0;
}
extern "C" int free_QED_temps(struct QED_kernel_temps*) { return 0; }
extern "C" void QED_Mkernel_L2(const double Lambda, const double xv[4], const double yv[4],
                               const struct QED_kernel_temps t, double kerv[6][4][4][4]) {
  if (!g_dense.empty()) {
    hlbl_qed_dense_kernel(g_dense.data(), xv, yv, kerv);
    return;
  }
  hlbl_qed_params p = t.p;
  p.lambda = Lambda;
  hlbl_qed_kernel(&p, xv, yv, kerv);
}
extern "C" void ref_set_qed_dense(int on, unsigned long long seed) {
  if (!on) {
    g_dense.clear();
    return;
  }
  g_dense.assign((std::size_t)HLBL_QED_DENSE_NB * HLBL_QED_NK, 0.0);
  hlbl_qed_dense_init(g_dense.data(), seed);
}

namespace {
Coord coord(const int v[4]) { return Coord{v[0], v[1], v[2], v[3]}; }
Geom geom(const int v[4]) { return Geom{v[0], v[1], v[2], v[3]}; }
}  // namespace

extern "C" {

// Contractor::kernel_sum on one rank with lattice `local` (= global).
int ref_kernel_sum(const int local[4], const double* src, const double* y, const int gsx[4],
                   const int yv[4], double xunit, double out[2]) {
  try {
    hlbl::Lattice lat(MPI_COMM_WORLD, hlbl::Vec4{1, 1, 1, 1},
                      hlbl::Vec4{local[0], local[1], local[2], local[3]});
    QED_kernel_temps kq;
    initialise(&kq);
    std::size_t const n = hlbl::block_length(lat);
    hlbl::DeviceBuffer<double> d_src(n), d_y(n);
    d_src.copy_from_host(src, n);
    d_y.copy_from_host(y, n);
    hlbl::Contractor c(lat, kq);
    auto r = c.kernel_sum(d_src.get(), d_y.get(), hlbl::Vec4{gsx[0], gsx[1], gsx[2], gsx[3]},
                          hlbl::Vec4{yv[0], yv[1], yv[2], yv[3]}, xunit);
    out[0] = r[0];
    out[1] = r[1];
    return 0;
  } catch (...) {
    return 1;
  }
}

// cu_dzu_dzsu with an arbitrary rank position (adds into dzu, dzsu).
void ref_dzu_dzsu(double* dzu, double* dzsu, const double* src, const double* y, int f,
                  const int pc[4], const int gsx[4], const int global[4], const int local[4]) {
  cu_dzu_dzsu(dzu, dzsu, src, y, f, coord(pc), coord(gsx), geom(global), geom(local));
}

// cu_4pt_contraction with an arbitrary rank position (adds into *ks).
void ref_4pt(double* ks, const double* g_dzu, const double* g_dzsu, const double* src,
             const double* y, int f, const int pc[4], const int gsx[4], double xunit,
             const int yv[4], const int global[4], const int local[4]) {
  QED_kernel_temps kq;
  initialise(&kq);
  cu_4pt_contraction(ks, g_dzu, g_dzsu, src, y, f, coord(pc), coord(gsx), Pair{xunit, 0.0},
                     coord(yv), kq, geom(global), geom(local));
}

// Contractor::pieces_2p2 on one rank with lattice `local` (= global):
// p1 [4][4][4][Lmax], p234 [n_y][5][64] (contract.cpp:116-156).
int ref_pieces_2p2(const int local[4], const double* fwd, const int gsw[4], const int* targets,
                   int n_y, double xunit, double* p1, double* p234) {
  try {
    hlbl::Lattice lat(MPI_COMM_WORLD, hlbl::Vec4{1, 1, 1, 1},
                      hlbl::Vec4{local[0], local[1], local[2], local[3]});
    QED_kernel_temps kq;
    initialise(&kq);
    std::size_t const n = hlbl::block_length(lat);
    hlbl::DeviceBuffer<double> d(n);
    d.copy_from_host(fwd, n);
    hlbl::Contractor c(lat, kq);
    std::vector<hlbl::Vec4> t;
    for (int i = 0; i < n_y; ++i)
      t.push_back(hlbl::Vec4{targets[4 * i], targets[4 * i + 1], targets[4 * i + 2], targets[4 * i + 3]});
    auto r = c.pieces_2p2(d.get(), hlbl::Vec4{gsw[0], gsw[1], gsw[2], gsw[3]}, t, xunit);
    std::copy(r.p1.begin(), r.p1.end(), p1);
    std::copy(r.p234.begin(), r.p234.end(), p234);
    return 0;
  } catch (...) {
    return 1;
  }
}

// compute_2p2_gpu (kernels.cu:753-870) of one rank at position pc: that
// rank's partial p1 [4][4][4][Lmax] and p234 [5][n_y][64] (the single-rank
// MPI shim leaves the all-reduce to the caller).
void ref_compute_2p2(const double* fwd, int iflavor, const int gsw[4], const int* targets, int n_y,
                     double xunit, const int pc[4], const int global[4], const int local[4],
                     double* p1, double* p234) {
  QED_kernel_temps kq;
  initialise(&kq);
  double const xu[2] = {xunit, 0.0};
  unsigned const vol = (unsigned)(local[0] * local[1] * local[2] * local[3]);
  compute_2p2_gpu(const_cast<double*>(fwd), p1, p234, iflavor, gsw, targets, n_y, xu, kq, vol, pc,
                  MPI_COMM_WORLD, local[0], local[1], local[2], local[3], global[0], global[1],
                  global[2], global[3]);
}

void ref_fill_random_block(const int local[4], std::uint64_t seed, double* out) {
  hlbl::Lattice lat(MPI_COMM_WORLD, hlbl::Vec4{1, 1, 1, 1},
                    hlbl::Vec4{local[0], local[1], local[2], local[3]});
  hlbl::fill_random_block(lat, seed, out);
}

// RandomProvider::compute: the block of the source at gsx.
void ref_random_provider(const int local[4], std::uint64_t seed, const int gsx[4], double* out) {
  hlbl::Lattice lat(MPI_COMM_WORLD, hlbl::Vec4{1, 1, 1, 1},
                    hlbl::Vec4{local[0], local[1], local[2], local[3]});
  hlbl::RandomProvider prov(lat, seed);
  hlbl::DeviceBuffer<double> d(hlbl::block_length(lat));
  prov.compute(hlbl::Vec4{gsx[0], gsx[1], gsx[2], gsx[3]}, d);
  d.copy_to_host(out, hlbl::block_length(lat));
}

void ref_apply_gamma(int g, const double* in, double* out) {
  hlbl::Spinor24 t;
  for (int i = 0; i < 24; ++i) t[i] = in[i];
  hlbl::Spinor24 s = hlbl::apply_gamma(g, t);
  for (int i = 0; i < 24; ++i) out[i] = s[i];
}

// build_schedule + all_pairs: rows (older[4], newer[4], window). Returns the
// number of pairs, or -1 if max_pairs is too small.
int ref_schedule_pairs(const int h[4], int stride, int n_steps, const int origin[4], int* out,
                       int max_pairs) {
  auto steps = hlbl::build_schedule(hlbl::Vec4{h[0], h[1], h[2], h[3]}, stride, n_steps,
                                    hlbl::Vec4{origin[0], origin[1], origin[2], origin[3]});
  int n = 0;
  for (const auto& st : steps)
    for (const auto& src : st.sources)
      for (const auto& q : src.partners) {
        if (n >= max_pairs) return -1;
        int* r = out + 9 * n;
        for (int i = 0; i < 4; ++i) r[i] = q[i];
        for (int i = 0; i < 4; ++i) r[4 + i] = src.position[i];
        r[8] = st.index;
        ++n;
      }
  return n;
}

// plan_2p2 + report_2p2 over n chains (chain c = build_schedule(h[c], stride,
// n_steps, origin[c])). Rows: at (chain, position[4], index), not_sources
// (site[4], chain, window), unsolved (index); the report's lines joined by
// newlines into `report` (cap bytes). Returns -1 if a buffer is too small.
int ref_plan_2p2(int n_chains, const int* h, int stride, int n_steps, const int* origin, int n_src,
                 const int* sources, const int lattice[4], int* at, int max_at, int* n_at, int* not_src,
                 int max_not, int* n_not, int* unsolved, int max_uns, int* n_uns, char* report,
                 int cap) {
  std::vector<hlbl::Schedule> chains;
  for (int c = 0; c < n_chains; ++c)
    chains.push_back(hlbl::build_schedule(hlbl::Vec4{h[4 * c], h[4 * c + 1], h[4 * c + 2], h[4 * c + 3]},
                                          stride, n_steps,
                                          hlbl::Vec4{origin[4 * c], origin[4 * c + 1], origin[4 * c + 2],
                                                     origin[4 * c + 3]}));
  std::vector<hlbl::Vec4> src;
  for (int i = 0; i < n_src; ++i)
    src.push_back(hlbl::Vec4{sources[4 * i], sources[4 * i + 1], sources[4 * i + 2], sources[4 * i + 3]});
  hlbl::Plan2p2 const plan =
      hlbl::plan_2p2(chains, src, hlbl::Vec4{lattice[0], lattice[1], lattice[2], lattice[3]});
  int k = 0;
  for (int c = 0; c < n_chains; ++c)
    for (const auto& [pos, idx] : plan.at[c]) {
      if (k >= max_at) return -1;
      int* r = at + 6 * k++;
      r[0] = c;
      for (int i = 0; i < 4; ++i) r[1 + i] = pos[i];
      r[5] = idx;
    }
  *n_at = k;
  k = 0;
  for (const auto& [p, c, w] : plan.not_sources) {
    if (k >= max_not) return -1;
    int* r = not_src + 6 * k++;
    for (int i = 0; i < 4; ++i) r[i] = p[i];
    r[4] = c;
    r[5] = w;
  }
  *n_not = k;
  if ((int)plan.unsolved.size() > max_uns) return -1;
  for (std::size_t i = 0; i < plan.unsolved.size(); ++i) unsolved[i] = plan.unsolved[i];
  *n_uns = (int)plan.unsolved.size();
  std::string all;
  for (const auto& line : hlbl::report_2p2(plan, src)) all += line + "\n";
  if ((int)all.size() + 1 > cap) return -1;
  std::copy(all.begin(), all.end(), report);
  report[all.size()] = 0;
  return 0;
}

// simulate(kInterleaved): propagators, pairs, peak cache.
void ref_schedule_stats(const int h[4], int stride, int n_steps, long long out[3]) {
  auto steps = hlbl::build_schedule(hlbl::Vec4{h[0], h[1], h[2], h[3]}, stride, n_steps);
  auto st = hlbl::simulate(steps, hlbl::Mode::kInterleaved);
  out[0] = st.n_propagators;
  out[1] = st.n_pairs;
  out[2] = st.peak_cache;
}

}  // extern "C"
