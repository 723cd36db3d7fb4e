// p1_f32.cu -- pass 1 (ker_dzu_dzsu, cuda_lattice.cu:160-262) of the mixed
// path on FP32 tile copies of the blocks (the layout of f32_tile_off): the
// blocks are converted once, when they enter the propagator cache
// (hlbl_f32_tile_copy), instead of in every pair's pass 1, so pass 1 reads
// half the bytes and converts nothing.
//
// The same arithmetic as p1_kernel<float, 2, TS>: thread (fl, ia, ib) forms
// per site the eight spin-block products of src[fl][ia] and y[1-fl][ib],
// X_sigma, and adds them into dzsu[sigma] and, weighted by the zerohalf
// coordinates, dzu[k]; per-tile FP32 sums go into Kahan FP32 accumulators,
// converted to FP64 at the end; partials per CTA in p1_kernel's layout.
// A tile is half of a 32-site tile of the copy (16 sites): one 1.5 KB TMA
// copy per row. NFL = 2: a CTA of 288 threads takes both flavours (48 rows);
// ST = 1: one stage, two CTAs per SM (the other CTA computes while one
// waits); ST = 2: two stages (the next tile prefetched while this one is
// computed), one CTA per SM. NFL = 1: a CTA of 144 threads takes one flavour
// (blockIdx.y = 2 pair + flavour, 24 rows), two stages, three CTAs per SM.
#include <cuda_runtime.h>

#include <cstdint>

#include "contract_kernels.cuh"
#include "hlbl_gb300.h"
#include "hlbl_internal.h"
#include "p2_tc.h"

namespace hg {
namespace p1f {

constexpr int kTS = 16;                   // sites per tile (half of a copy tile)
constexpr int kRowFloats = kTS * 24;      // 384: [c4][16][4]
constexpr uint32_t kRowBytes = kRowFloats * 4;
// staged rows 16 bytes apart more than their length, so that the rows the
// threads of one warp read (12 y rows, 3 x rows) start in different banks
constexpr int kRowStride = kRowFloats + 4;
template <int NFL> __host__ __device__ constexpr int rows() { return 24 * NFL; }   // (x, y) x flavours x 12
template <int NFL> __host__ __device__ constexpr int threads() { return 144 * NFL; }
template <int ST, int NFL> __host__ __device__ constexpr int min_ctas() { return NFL == 1 ? 3 : (ST == 1 ? 2 : 1); }

// One tile's contribution of thread (fl, ia, ib): per site the eight
// spin-block products and X_sigma; added into the Kahan accumulators.
// The zerohalf weights zh_0..zh_2 are constant along a run of sites of
// fixed (t, x, y) (z fastest), so per site only the run sums S_g = sum X_g and
// T_g = sum zh_3 X_g are formed, and at the end of a run
//   dzu[(r,g)] += zh_r S_g - zh_g S_r  (g < 3),   zh_r S_3 - T_r  (g = 3),
//   dzsu[g]    += S_g.
// z0: the tile's first site's local z, LZ: the local extent in z.
__device__ __forceinline__ void tile_sums(const float* __restrict__ Arow, const float* __restrict__ Brow,
                                          const float (*zhs)[4], int nvalid, int z0, int LZ,
                                          KahanF (&acc_u)[6][2], KahanF (&acc_s)[4][2]) {
  float tu[6][2], ts[4][2], S[4][2], T[4][2];
#pragma unroll
  for (int k = 0; k < 6; ++k) tu[k][0] = tu[k][1] = 0.f;
#pragma unroll
  for (int g = 0; g < 4; ++g) ts[g][0] = ts[g][1] = S[g][0] = S[g][1] = T[g][0] = T[g][1] = 0.f;
  auto flush = [&](const float* zh) {
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      int const r = comb_rho(k), g = comb_sigma(k);
#pragma unroll
      for (int c = 0; c < 2; ++c)
        tu[k][c] += g == 3 ? zh[r] * S[3][c] - T[r][c] : zh[r] * S[g][c] - zh[g] * S[r][c];
    }
#pragma unroll
    for (int g = 0; g < 4; ++g) {
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        ts[g][c] += S[g][c];
        S[g][c] = T[g][c] = 0.f;
      }
    }
  };
  int z = z0;
#pragma unroll 1
  for (int s = 0; s < nvalid; ++s) {
    if (z == LZ) {  // a new run starts at this site
      flush(zhs[s - 1]);
      z = 0;
    }
    ++z;
    float A[24], B[24];
#pragma unroll
    for (int c4 = 0; c4 < 6; ++c4) {
      float4 const a = *reinterpret_cast<const float4*>(Arow + c4 * 64 + s * 4);
      float4 const b = *reinterpret_cast<const float4*>(Brow + c4 * 64 + s * 4);
      A[4 * c4] = a.x; A[4 * c4 + 1] = a.y; A[4 * c4 + 2] = a.z; A[4 * c4 + 3] = a.w;
      B[4 * c4] = b.x; B[4 * c4 + 1] = b.y; B[4 * c4 + 2] = b.z; B[4 * c4 + 3] = b.w;
    }
    // P[s1][s2] = sum_c conj(B[s1][c]) A[s2][c] for s2 = s1^2 and 3-s1, as
    // packed FP32 pairs: with y = (Re B, Im B), U = sum_c y Re A and
    // V = sum_c y Im A (the A part broadcast to both halves), Re P = U.x + V.y
    // and Im P = V.x - U.y -- two packed FMAs per (c, s2) instead of four
    float pa[4][2], pb[4][2];
#pragma unroll
    for (int s1 = 0; s1 < 4; ++s1) {
      float2 ua = make_float2(0.f, 0.f), va = ua, ub = ua, vb = ua;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float2 const y = make_float2(B[2 * (3 * s1 + c)], B[2 * (3 * s1 + c) + 1]);
        int const sa = 2 * (3 * (s1 ^ 2) + c), sb = 2 * (3 * (3 - s1) + c);
        ua = __ffma2_rn(y, make_float2(A[sa], A[sa]), ua);
        va = __ffma2_rn(y, make_float2(A[sa + 1], A[sa + 1]), va);
        ub = __ffma2_rn(y, make_float2(A[sb], A[sb]), ub);
        vb = __ffma2_rn(y, make_float2(A[sb + 1], A[sb + 1]), vb);
      }
      pa[s1][0] = ua.x + va.y; pa[s1][1] = va.x - ua.y;
      pb[s1][0] = ub.x + vb.y; pb[s1][1] = vb.x - ub.y;
    }
    float const z3 = zhs[s][3];
#pragma unroll
    for (int sg = 0; sg < 4; ++sg) {
      float xr = 0, xi = 0;
#pragma unroll
      for (int s1 = 0; s1 < 4; ++s1) {
        float const* pp = (sg == 0 || sg == 3) ? pa[s1] : pb[s1];
        float vr, vi;
        mul_iph(g5g_ph(sg, s1), pp[0], pp[1], vr, vi);
        xr += vr; xi += vi;
      }
      S[sg][0] += xr; S[sg][1] += xi;
      T[sg][0] = fmaf(z3, xr, T[sg][0]); T[sg][1] = fmaf(z3, xi, T[sg][1]);
    }
  }
  if (nvalid > 0) flush(zhs[nvalid - 1]);
#pragma unroll
  for (int k = 0; k < 6; ++k) { acc_u[k][0].add(tu[k][0]); acc_u[k][1].add(tu[k][1]); }
#pragma unroll
  for (int g = 0; g < 4; ++g) { acc_s[g][0].add(ts[g][0]); acc_s[g][1].add(ts[g][1]); }
}

template <int ST, int NFL>
struct Smem {
  float stage[ST][rows<NFL>()][kRowStride];
  float zh[2][kTS][4];  // this tile's zero-half weights and the next one's
};

template <int ST, int NFL>
__global__ void __launch_bounds__(threads<NFL>(), min_ctas<ST, NFL>())
p1f32_kernel(TcBatch tb, Geometry geo, double* __restrict__ partials, int* __restrict__ err) {
  constexpr int kRows = rows<NFL>();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<ST, NFL>& sm = *reinterpret_cast<Smem<ST, NFL>*>(smem_raw);
  __shared__ __align__(8) uint64_t s_bar[ST];
  __shared__ int s_fail;
  int const t = threadIdx.x;
  // NFL = 1: blockIdx.y = 2 pair + flavour; the CTA's rows are that flavour's
  int const pi = NFL == 1 ? blockIdx.y >> 1 : blockIdx.y;
  int const fl = NFL == 1 ? (int)(blockIdx.y & 1) : t / 144;
  int const ia = (t % 144) / 12, ib = t % 12;
  const float* __restrict__ x32 = tb.x32[pi];
  const float* __restrict__ y32 = tb.y32;
  int const gsx[4] = {tb.gsx[pi][0], tb.gsx[pi][1], tb.gsx[pi][2], tb.gsx[pi][3]};
  long long const nt32 = (geo.V + 31) / 32;
  long long const ntiles = (geo.V + kTS - 1) / kTS;
  // rows: which = 0 x at flavour fl, which = 1 y at flavour 1 - fl
  // (NFL = 2: [which][f][12]; NFL = 1: [which][12] of the CTA's flavour)
  auto issue = [&](long long tile, int st) {
    mbar_arrive_expect_tx(&s_bar[st], kRows * kRowBytes);
    long long const t32 = tile >> 1, half = tile & 1;
    for (int row = 0; row < kRows; ++row) {
      int const which = row / (12 * NFL), f = NFL == 1 ? fl : (row / 12) % 2, i = row % 12;
      int const ff = which == 0 ? f : 1 - f;
      const float* src = (which == 0 ? x32 : y32) + ((size_t)(ff * 12 + i) * nt32 + t32) * kRowF32 + half * kRowFloats;
      bulk_g2s(sm.stage[st][row], src, kRowBytes, &s_bar[st]);
    }
  };
  if (t == 0) {
    for (int i = 0; i < ST; ++i) mbar_init(&s_bar[i], 1);
    fence_mbar_init();
    s_fail = 0;
  }
  __syncthreads();

  KahanF acc_u[6][2], acc_s[4][2];
  // a tile's zero-half weights, a thread per site (its four), with 32-bit
  // index arithmetic where the volume allows it
  bool const small = geo.V <= 0xFFFFFFFFLL;
  auto zh_fill = [&](long long tl, int buf) {
    long long const s0 = tl * kTS;
    for (int s = t; s < kTS; s += blockDim.x) {
      int rel[4];
      rel_coords_fast(geo, gsx, min(s0 + s, geo.V - 1), rel);
#pragma unroll
      for (int r = 0; r < 4; ++r) sm.zh[buf][s][r] = (float)coord_map_zerohalf(rel[r], geo.global[r]);
    }
  };
  long long tile = blockIdx.x;
  if (tile < ntiles) {
    if (t == 0) issue(tile, 0);
    zh_fill(tile, 0);
  }
  __syncthreads();
  // one block barrier per tile: the next tile's weights are written (into the
  // other zh buffer) before it, and the stage and zh buffer of this tile are
  // rewritten only after the next one
  int it = 0;
  for (; tile < ntiles; tile += gridDim.x, ++it) {
    int const st = ST == 1 ? 0 : (it & 1), zb = it & 1;
    uint32_t const parity = ST == 1 ? (uint32_t)(it & 1) : (uint32_t)((it >> 1) & 1);
    bool const more = tile + gridDim.x < ntiles;
    // ST = 2: prefetch the next tile into the other stage (its readers passed
    // the previous iteration's barrier)
    if (ST == 2 && t == 0 && more) {
      fence_proxy_async_smem();
      issue(tile + gridDim.x, st ^ 1);
    }
    const float* Arow = sm.stage[st][NFL == 1 ? ia : fl * 12 + ia];
    const float* Brow = sm.stage[st][NFL == 1 ? 12 + ib : 24 + fl * 12 + ib];
    long long const s0 = tile * kTS;
    int const nvalid = (int)min((long long)kTS, geo.V - s0);
    int const z0 = small ? (int)((unsigned)s0 % (unsigned)geo.local[3]) : (int)(s0 % geo.local[3]);
    if (mbar_wait(&s_bar[st], parity)) tile_sums(Arow, Brow, sm.zh[zb], nvalid, z0, geo.local[3], acc_u, acc_s);
    else s_fail = 1;
    if (more) zh_fill(tile + gridDim.x, zb ^ 1);
    __syncthreads();  // the stage and zh[zb] are rewritten after this
    if (s_fail) break;
    if (ST == 1 && t == 0 && more) {
      fence_proxy_async_smem();
      issue(tile + gridDim.x, 0);
    }
  }
  if (s_fail) {
    // a wait gave up: report it and let the copy it waited for (the only
    // one in flight) land before the CTA exits (bounded, as everything else)
    if (t == 0) {
      if (err) atomicExch(err, kErrWaitTimeout);
      int const st = ST == 1 ? 0 : (it & 1);
      mbar_wait(&s_bar[st], ST == 1 ? (uint32_t)(it & 1) : (uint32_t)((it >> 1) & 1));
      if (ST == 2 && tile + gridDim.x < ntiles)
        mbar_wait(&s_bar[st ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
    }
    return;
  }
  double* out = partials + (((size_t)pi * gridDim.x + blockIdx.x) * 2 + fl) * kDzLen;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    out[((k * 12 + ia) * 12 + ib) * 2] = acc_u[k][0].get();
    out[((k * 12 + ia) * 12 + ib) * 2 + 1] = acc_u[k][1].get();
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    out[kDzuLen + ((s * 12 + ia) * 12 + ib) * 2] = acc_s[s][0].get();
    out[kDzuLen + ((s * 12 + ia) * 12 + ib) * 2 + 1] = acc_s[s][1].get();
  }
}


// ---- warp-specialized form (variant 3): one flavour per CTA, a producer
// warp and empty/full mbarriers per stage instead of a block barrier per tile.
// Warps 0-4 compute (threads 0..143, (ia, ib)); warp 5 computes each tile's
// zerohalf weights and issues its TMA copies. A stage is refilled once all
// five compute warps have released it, so a warp may run a tile ahead.
constexpr int kWsStages = 2;
constexpr int kWsThreads = 192;
constexpr int kWsComputeWarps = 5;

struct SmemWs {
  float stage[kWsStages][24][kRowStride];
  float zh[kWsStages][kTS][4];
};

__device__ __forceinline__ void mbar_arrive_local(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// three CTAs of 192 threads per SM: at most 104 registers a thread
__global__ void __maxnreg__(104)
p1f32_ws_kernel(TcBatch tb, Geometry geo, double* __restrict__ partials, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemWs& sm = *reinterpret_cast<SmemWs*>(smem_raw);
  __shared__ __align__(8) uint64_t s_full[kWsStages], s_empty[kWsStages];
  __shared__ int s_fail;
  int const t = threadIdx.x, warp = t >> 5, lane = t & 31;
  int const pi = blockIdx.y >> 1, fl = (int)(blockIdx.y & 1);
  int const ia = (t % 144) / 12, ib = t % 12;
  long long const ntiles = (geo.V + kTS - 1) / kTS;
  if (t == 0) {
    for (int i = 0; i < kWsStages; ++i) {
      mbar_init(&s_full[i], 32);  // the producer warp's lanes (lane 0 with the bytes)
      mbar_init(&s_empty[i], kWsComputeWarps);
    }
    fence_mbar_init();
    s_fail = 0;
  }
  __syncthreads();
  volatile int* fail = &s_fail;
  KahanF acc_u[6][2], acc_s[4][2];
  long long last[kWsStages] = {-1, -1};  // producer: the last tile issued into each stage
  if (warp == kWsComputeWarps) {
    // ---- producer ----
    const float* __restrict__ x32 = tb.x32[pi];
    const float* __restrict__ y32 = tb.y32;
    int const gsx[4] = {tb.gsx[pi][0], tb.gsx[pi][1], tb.gsx[pi][2], tb.gsx[pi][3]};
    long long const nt32 = (geo.V + 31) / 32;
    int it = 0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      int const st = it % kWsStages;
      // stage st is free once the five compute warps released its previous tile
      if (it >= kWsStages && !mbar_wait(&s_empty[st], (uint32_t)((it / kWsStages - 1) & 1))) {
        *fail = 1;
        break;
      }
      if (*fail) break;
      long long const s0 = tile * kTS;
      for (int s = lane; s < kTS; s += 32) {
        int rel[4];
        rel_coords_fast(geo, gsx, min(s0 + s, geo.V - 1), rel);
#pragma unroll
        for (int r = 0; r < 4; ++r) sm.zh[st][s][r] = (float)coord_map_zerohalf(rel[r], geo.global[r]);
      }
      if (lane == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&s_full[st], 24 * kRowBytes);
        long long const t32 = tile >> 1, half = tile & 1;
        for (int row = 0; row < 24; ++row) {
          int const which = row / 12, i = row % 12, ff = which == 0 ? fl : 1 - fl;
          const float* src = (which == 0 ? x32 : y32) + ((size_t)(ff * 12 + i) * nt32 + t32) * kRowF32 +
                             half * kRowFloats;
          bulk_g2s(sm.stage[st][row], src, kRowBytes, &s_full[st]);
        }
        last[st] = it;
      } else {
        mbar_arrive_local(&s_full[st]);  // releases this lane's zero-half weights
      }
    }
  } else {
    // ---- compute warps ----
    int it = 0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      int const st = it % kWsStages;
      if (!mbar_wait(&s_full[st], (uint32_t)((it / kWsStages) & 1))) {
        *fail = 1;
        break;
      }
      if (*fail) break;
      if (t < 144) {
        long long const s0 = tile * kTS;
        int const nvalid = (int)min((long long)kTS, geo.V - s0);
        tile_sums(sm.stage[st][ia], sm.stage[st][12 + ib], sm.zh[st], nvalid, (int)(s0 % geo.local[3]),
                  geo.local[3], acc_u, acc_s);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive_local(&s_empty[st]);
    }
  }
  __syncthreads();
  if (*fail) {
    // a wait gave up: report it; the producer lets every copy in flight land
    // before the CTA exits (bounded)
    if (t == 0 && err) atomicExch(err, kErrWaitTimeout);
    if (warp == kWsComputeWarps && lane == 0)
      for (int st = 0; st < kWsStages; ++st)
        if (last[st] >= 0) mbar_wait(&s_full[st], (uint32_t)((last[st] / kWsStages) & 1));
    return;
  }
  if (t >= 144) return;
  double* out = partials + (((size_t)pi * gridDim.x + blockIdx.x) * 2 + fl) * kDzLen;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    out[((k * 12 + ia) * 12 + ib) * 2] = acc_u[k][0].get();
    out[((k * 12 + ia) * 12 + ib) * 2 + 1] = acc_u[k][1].get();
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    out[kDzuLen + ((s * 12 + ia) * 12 + ib) * 2] = acc_s[s][0].get();
    out[kDzuLen + ((s * 12 + ia) * 12 + ib) * 2 + 1] = acc_s[s][1].get();
  }
}

}  // namespace p1f

template <int ST, int NFL>
int p1f32_init_t(int nsm, int& grid) {
  size_t const smem = sizeof(p1f::Smem<ST, NFL>);
  cudaError_t e = cudaFuncSetAttribute(p1f::p1f32_kernel<ST, NFL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(p1f::p1f32_kernel<ST, NFL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return cuda_fail(e, "p1f32 smem attribute");
  int nb = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, p1f::p1f32_kernel<ST, NFL>, p1f::threads<NFL>(), smem);
  if (e != cudaSuccess) return cuda_fail(e, "p1f32 occupancy");
  if (nb < 1) return fail(HLBL_ECUDA, "p1f32 kernel cannot be resident");
  // NFL = 1 launches two CTAs (one per flavour) per tile range: the same
  // number of CTAs per pair as NFL = 2 at its occupancy
  grid = NFL == 1 ? (nb * nsm) / 2 : nb * nsm;
  return HLBL_OK;
}

int p1f32_init_ws(int nsm, int& grid) {
  size_t const smem = sizeof(p1f::SmemWs);
  cudaError_t e = cudaFuncSetAttribute(p1f::p1f32_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(p1f::p1f32_ws_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return cuda_fail(e, "p1f32 smem attribute");
  int nb = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, p1f::p1f32_ws_kernel, p1f::kWsThreads, smem);
  if (e != cudaSuccess) return cuda_fail(e, "p1f32 occupancy");
  if (nb < 1) return fail(HLBL_ECUDA, "p1f32 kernel cannot be resident");
  grid = (nb * nsm) / 2;  // two CTAs (one per flavour) per tile range
  return HLBL_OK;
}

int p1f32_init(int nsm, int grid[kP1f32Variants]) {
  if (int rc = p1f32_init_t<1, 2>(nsm, grid[0])) return rc;
  if (int rc = p1f32_init_t<2, 2>(nsm, grid[1])) return rc;
  if (int rc = p1f32_init_t<2, 1>(nsm, grid[2])) return rc;
  return p1f32_init_ws(nsm, grid[3]);
}

long long p1f32_tiles(long long V) { return (V + p1f::kTS - 1) / p1f::kTS; }

void p1f32_launch(int variant, int grid, int npairs, cudaStream_t st, const TcBatch& tb, const Geometry& geo,
                  double* partials, int* err) {
  if (variant == 0)
    p1f::p1f32_kernel<1, 2><<<dim3(grid, npairs), p1f::threads<2>(), sizeof(p1f::Smem<1, 2>), st>>>(tb, geo, partials, err);
  else if (variant == 1)
    p1f::p1f32_kernel<2, 2><<<dim3(grid, npairs), p1f::threads<2>(), sizeof(p1f::Smem<2, 2>), st>>>(tb, geo, partials, err);
  else if (variant == 2)
    p1f::p1f32_kernel<2, 1><<<dim3(grid, 2 * npairs), p1f::threads<1>(), sizeof(p1f::Smem<2, 1>), st>>>(tb, geo, partials, err);
  else
    p1f::p1f32_ws_kernel<<<dim3(grid, 2 * npairs), p1f::kWsThreads, sizeof(p1f::SmemWs), st>>>(tb, geo, partials, err);
}

}  // namespace hg
