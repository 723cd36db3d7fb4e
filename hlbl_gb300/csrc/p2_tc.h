// p2_tc.h -- the tensor-core pass 2 (p2_tc.cu) as seen by the context code.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "contract_kernels.cuh"

namespace hg {

// FP32 tile copies of a propagator block, written by pass 1 (FP32 path) and
// read by the tensor-core pass 2: [f][ia][tile][6][32][4] floats, tiles of
// 32 sites (the last one padded), a site's 24 sink components as six
// 16-byte groups.
constexpr int kTileSites32 = 32;
constexpr int kRowF32 = kTileSites32 * 24;
inline size_t f32_block_floats(long long V) {
  return (size_t)2 * 12 * (size_t)((V + kTileSites32 - 1) / kTileSites32) * kRowF32;
}

// The pairs of one tensor-core pass-2 launch (blockIdx.y = pair).
struct TcBatch {
  const float* y32;
  const float* x32[kMaxBatch];
  int gsx[kMaxBatch][4];
  int yv[kMaxBatch][4];
};

size_t tc_smem_bytes();
int tc_threads();
size_t tc_btu_floats_per_pair();
int tc_init(int nsm, int& grid);
void tc_launch_btu(const double* d_g, int npairs, float* d_btu, cudaStream_t st);
void tc_launch_p2(int grid, int npairs, cudaStream_t st, const TcBatch& tb, const Geometry& geo,
                  const P2Args& a, const float* d_btu, double* partials, int* err);
long long tc_tiles(long long V);

}  // namespace hg
