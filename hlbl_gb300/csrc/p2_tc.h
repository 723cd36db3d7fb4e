// p2_tc.h -- the tensor-core pass 2 (p2_tc.cu) as seen by the context code.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "contract_kernels.cuh"

namespace hg {

// FP32 tile copies of a propagator block, written by pass 1 (FP32 path) or
// hlbl_f32_tile_copy and read by the tensor-core pass 2 and the FP32-input
// pass 1: [f][ia][tile][2][6][16][4] floats (f32_tile_off), tiles of 32
// sites in two halves (the last tile padded), a site's 24 sink components as
// six 16-byte groups.
// A copy ends with a trailer of kF32Trailer floats: [0] and [1] hold the
// largest magnitude of flavour 0 and 1 (written by hlbl_f32_tile_copy; the
// FP16-operand pass 2 scales by them).
constexpr int kTileSites32 = 32;
constexpr int kRowF32 = kTileSites32 * 24;
constexpr int kF32Trailer = 32;
__host__ __device__ inline size_t f32_tile_floats(long long V) {
  return (size_t)2 * 12 * (size_t)((V + kTileSites32 - 1) / kTileSites32) * kRowF32;
}
inline size_t f32_block_floats(long long V) { return f32_tile_floats(V) + kF32Trailer; }

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
// f16: FP16 operands (B built with a per-(pair, flavour) scale into
// d_bscale[2 * pair + flavour]; the copies' trailers give A's scale)
void tc_launch_btu(const double* d_g, int npairs, void* d_btu, bool f16, float* d_bscale, cudaStream_t st);
void tc_launch_p2(int grid, int npairs, cudaStream_t st, const TcBatch& tb, const Geometry& geo,
                  const P2Args& a, const void* d_btu, bool f16, const float* d_bscale, double* partials, int* err);
long long tc_tiles(long long V);

// Pass 1 on FP32 tile copies (p1_f32.cu); partials in p1_kernel's layout.
// variant 0: both flavours per CTA, one stage, two CTAs per SM; 1: both
// flavours, two stages, one CTA per SM; 2: one flavour per CTA, two stages,
// three CTAs per SM; 3: as 2 with a producer warp and per-stage empty/full
// mbarriers instead of a block barrier per tile
constexpr int kP1f32Variants = 4;
int p1f32_init(int nsm, int grid[kP1f32Variants]);
long long p1f32_tiles(long long V);
void p1f32_launch(int variant, int grid, int npairs, cudaStream_t st, const TcBatch& tb, const Geometry& geo,
                  double* partials, int* err);

}  // namespace hg
