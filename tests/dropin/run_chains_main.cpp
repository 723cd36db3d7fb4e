// run_chains_main.cpp -- TEST INFRASTRUCTURE. A program over the reference's
// own driver: it builds the reference's Lattice, RandomProvider and
// Contractor and runs its run_chains (src/driver.cpp:169-208) on the
// configuration of sanity_check/test_driver_random.cpp:133-160 (6^4, h =
// (1,1,1,1), stride 1, two steps, four 2+2 sources), with the device cache
// and with the host cache, then writes every pair's kernel sums and every
// 2+2 source's pieces as JSON to the file argv[1] (the driver itself prints
// its progress on stdout). tests/dropin/Makefile links it twice: with the
// reference's own kernels, and with the library's drop-in launchers
// (hlbl_gb300/dropin) and libhlbl_gb300.so. Never shipped.
#include <cstdio>
#include <vector>

#include "hlbl/driver.hpp"
#include "hlbl/physics.hpp"

using namespace hlbl;

namespace {

std::FILE* g_out = nullptr;

void print_run(const char* name, const std::vector<PairResult>& rows, const std::vector<Result2p2>& r22,
               const RunStats& st) {
  std::fprintf(g_out, "{\"run\": \"%s\", \"pairs\": %d, \"cache_peak\": %d, \"positions_solved\": %d,\n", name,
              st.pairs, st.cache_peak, st.positions_solved);
  std::fprintf(g_out, " \"kernel_sums\": [");
  for (std::size_t i = 0; i < rows.size(); ++i) {
    const PairResult& r = rows[i];
    std::fprintf(g_out, "%s[[%d,%d,%d,%d],[%d,%d,%d,%d],%d,%d,%.17g,%.17g]", i ? ",\n  " : "", r.x[0], r.x[1], r.x[2],
                r.x[3], r.y[0], r.y[1], r.y[2], r.y[3], r.chain, r.window, r.kernel_sum[0], r.kernel_sum[1]);
  }
  std::fprintf(g_out, "],\n \"pieces_2p2\": [");
  for (std::size_t i = 0; i < r22.size(); ++i) {
    std::fprintf(g_out, "%s{\"w\": [%d,%d,%d,%d], \"p1\": [", i ? ",\n  " : "", r22[i].w[0], r22[i].w[1], r22[i].w[2],
                r22[i].w[3]);
    for (std::size_t k = 0; k < r22[i].p1.size(); ++k) std::fprintf(g_out, "%s%.17g", k ? "," : "", r22[i].p1[k]);
    std::fprintf(g_out, "], \"p234\": [");
    for (std::size_t k = 0; k < r22[i].p234.size(); ++k) std::fprintf(g_out, "%s%.17g", k ? "," : "", r22[i].p234[k]);
    std::fprintf(g_out, "]}");
  }
  std::fprintf(g_out, "]}\n");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2 || !(g_out = std::fopen(argv[1], "w"))) return 2;
  MPI_Init(&argc, &argv);
  Lattice lat(MPI_COMM_WORLD, Vec4{1, 1, 1, 1}, Vec4{6, 6, 6, 6});
  Vec4 const h{1, 1, 1, 1};
  Schedule const schedule = build_schedule(h, 1, 2);
  std::vector<Source2p2> const sources_2p2 = {
      {Vec4{0, 0, 0, 0}, {Vec4{3, 3, 3, 3}, Vec4{0, 5, 1, 2}}, 1},
      {Vec4{1, 1, 1, 1}, {Vec4{0, 0, 0, 0}}, 2},
      {Vec4{2, 2, 2, 2}, {Vec4{5, 5, 5, 5}, Vec4{1, 1, 1, 1}, Vec4{3, 0, 4, 1}}, 3}};
  QED_kernel_temps kqed_t;
  if (initialise(&kqed_t) != 0) return 1;
  Contractor contractor(lat, kqed_t);
  RandomProvider provider(lat, 7);
  RunOptions opt;
  opt.xunit = xunit(105.6583745, 0.07957);
  opt.sources_2p2 = sources_2p2;
  std::fprintf(g_out, "[\n");
  for (int host = 0; host < 2; ++host) {
    RunOptions o = opt;
    if (host) o.residency = PropagatorCache::Residency::kHost;
    RunStats st;
    std::vector<Result2p2> r22;
    auto rows = run_chains(lat, {schedule}, o, provider, contractor, nullptr, nullptr, &st, &r22);
    print_run(host ? "host_cache" : "device_cache", rows, r22, st);
    if (!host) std::fprintf(g_out, ",\n");
  }
  std::fprintf(g_out, "]\n");
  std::fclose(g_out);
  MPI_Finalize();
  return 0;
}
