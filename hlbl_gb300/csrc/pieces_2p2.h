// pieces_2p2.h -- the 2+2 pieces (pieces_2p2.cu) as seen by the context code.
#pragma once

#include <cuda_runtime.h>

#include "hlbl_device.cuh"
#include "qed_f32.cuh"

namespace hg {

// targets per launch of the per-target kernels (more are done in chunks)
constexpr int kMaxTargets = 32;

// Kernel parameters of the per-target kernels.
struct P234Args {
  Geometry geo;
  int gsw[4];
  int n_t;                  // targets of this launch
  int y[kMaxTargets][4];    // (target - gsw) mod G
  double xunit;
  float r64f;               // FP32 path: FP64 weight where |a| or |b| < r64 (0: nowhere)
  hlbl_qed_params qp;
  QedF32 qf;
};

struct P22Request {
  const double* fwd;        // device block of the source w
  const float* x32;         // or (FP32 path) its FP32 tile copy; null: use fwd
  int iflavor;
  int gsw[4];
  const int* targets;       // host, [n_y][4], global sites in [0, L)
  int n_y;
  double xunit;
  int precision;            // HLBL_FP64 | HLBL_FP32
  double r64;
  double* d_p1;             // device [4][4][4][Lmax]
  double* d_p234;           // device, [n_y][5][64] or (raw_layout) [5][n_y][64]
  int raw_layout;
};

struct P22;
int p22_reserve(P22** st, const Geometry& geo, int nsm);
struct QedSel;
int p22_run(P22** st, cudaStream_t stream, const Geometry& geo, const QedSel& q, int nsm,
            bool capturing, const P22Request& rq);
void p22_destroy(P22* st);
int p22_lmax(const Geometry& geo);

}  // namespace hg
