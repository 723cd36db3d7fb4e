// output_nohdf5.cpp -- TEST INFRASTRUCTURE. The reference's ResultWriter needs
// HDF5 (src/output.cpp), which this machine lacks; run_chains_main passes no
// writer and no timing log, but src/driver.cpp names their methods, so the
// link needs definitions. These do nothing. Never shipped.
#include "hlbl/output.hpp"

namespace hlbl {
ResultWriter::ResultWriter(const std::string&, const RunInfo&) {}
ResultWriter::~ResultWriter() = default;
void ResultWriter::append(const std::vector<PairResult>&) {}
void ResultWriter::append_2p2(const std::vector<Result2p2>&) {}
TimingLog::TimingLog(const std::string&) {}
TimingLog::~TimingLog() = default;
void TimingLog::solve(int, int, const Vec4&, double, int) {}
void TimingLog::kernel_sum(int, int, const Vec4&, const Vec4&, double) {}
void TimingLog::pieces_2p2(int, int, const Vec4&, double) {}
}  // namespace hlbl
