// contract_kernels.cuh -- the connected-contraction kernels (pass 1, the
// gamma insertion, pass 2) and their reductions, templated on the compute
// type T of the per-site spin-colour products (double: the exact path;
// float: the mixed path). Site and volume sums are FP64 in both.
//
// Data layout in HBM (the reference's, src/provider.cpp:45):
//   block[((f*12 + ia)*V + site)*24 + c], f flavour, ia source spin-colour,
//   c = 2*(3*spin + colour) + {re, im} at the sink.
// A tile of TS consecutive sites of one (f, ia) row is TS*192 contiguous
// bytes, so every tile load is a set of 48 contiguous 16-byte-aligned runs.
#pragma once

#include <type_traits>

#include "hlbl_device.cuh"
#include "qed_f32.cuh"

namespace hg {

constexpr int kDzLen = 2880;       // dzu[6][12][12][2] + dzsu[4][12][12][2]
constexpr int kDzuLen = 1728;
constexpr int kGLen = 11520;       // g_dzu[6][4][12][24] + g_dzsu[4][4][12][24]
constexpr int kGDzuLen = 6912;
constexpr int kBtK = 288;          // rows of Bt: (p, q, re/im)
constexpr int kBtN = 160;          // columns of Bt: (j, nu, lambda), j < 10

// Up to kMaxBatch pairs that share the block y (the pairs one new source
// closes), passed by value as a kernel parameter; a kernel's blockIdx.y is
// the pair. Partners run over the same tile sequence at the same time, so
// y's tiles come from HBM about once and from L2 for the others.
constexpr int kMaxBatch = 16;
struct PairDesc {
  const double* src;  // the partner's block (the pair's x = gsx)
  double* out;        // its two kernel sums (pass 2 reduction target)
  float* src32;       // FP32 path: pass 1 writes the block's FP32 tile copy here (or null)
  int gsx[4];
  int yv[4];
};
struct PairBatch {
  int n;
  PairDesc p[kMaxBatch];
};

// Neumaier's compensated FP64 sum: the site-block and volume sums.
struct Neu {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double v) {
    double const t = s + v;
    c += fabs(s) >= fabs(v) ? (s - t) + v : (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ double get() const { return s + c; }
};


// Input staging: FP64 kernels double-buffer the FP64 tile (TMA into one
// stage while computing on the other); FP32 kernels keep one FP64 stage and
// convert each landed tile once into an FP32 copy, then re-use the stage
// for the next tile's TMA while computing on the copy (an FP64 -> FP32
// conversion issues on the FP64 pipe, so converting at every use is slow).
// Row stride of a staged tile in the compute type: FP64 stages are the TMA
// target, TS*24 dense; the FP32 copy pads each row by 16 bytes, so that the
// rows threads of one warp read start in different banks.
template <typename T, int TS>
constexpr int row_stride() { return sizeof(T) == sizeof(double) ? TS * 24 : TS * 24 + 4; }

template <typename T, int NF, int TS>
constexpr size_t stage_bytes() {
  return sizeof(T) == sizeof(double)
             ? sizeof(double) * (size_t)(2 * 2 * NF * 12 * TS * 24)
             : sizeof(double) * (size_t)(2 * NF * 12 * TS * 24) +
                   sizeof(float) * (size_t)(2 * NF * 12 * row_stride<float, TS>());
}

// TMA staging of one tile: rows (which, fl, ia) of the two blocks, the
// tile's nvalid sites each (one contiguous run of nvalid*192 bytes per row),
// into `stage` [2*NF*12][TS][24] doubles; which = 0 reads `a` at flavour
// fa0 + fa_step*fl, which = 1 reads `b` at fb0 + fb_step*fl. One thread.
template <int NF, int TS>
__device__ __forceinline__ void issue_tile(double* stage, uint64_t* bar, const double* a,
                                           const double* b, int fa0, int fa_step, int fb0,
                                           int fb_step, long long V, long long s0) {
  constexpr int kRows = 2 * NF * 12;
  int const nvalid = (int)min((long long)TS, V - s0);
  uint32_t const bytes = (uint32_t)nvalid * 192u;
  mbar_arrive_expect_tx(bar, bytes * kRows);
  for (int row = 0; row < kRows; ++row) {
    int const which = row / (NF * 12), fl = (row / 12) % NF, ia = row % 12;
    int const f = which == 0 ? fa0 + fa_step * fl : fb0 + fb_step * fl;
    const double* src = (which == 0 ? a : b) + ((size_t)(f * 12 + ia) * V + s0) * 24;
    bulk_g2s(stage + (size_t)row * TS * 24, src, bytes, bar);
  }
}

// Convert a landed FP64 stage into the FP32 compute copy (all threads),
// rows at stride row_stride<float, TS>().
template <int NF, int TS>
__device__ __forceinline__ void convert_stage(const double* __restrict__ st, float* __restrict__ cp) {
  constexpr int kRowPairs = TS * 24 / 2, RS = row_stride<float, TS>();
  constexpr int kN = 2 * NF * 12 * kRowPairs;
  const double2* s2 = reinterpret_cast<const double2*>(st);
  for (int i = threadIdx.x; i < kN; i += blockDim.x) {
    double2 const v = s2[i];
    int const row = i / kRowPairs, k = i % kRowPairs;
    *reinterpret_cast<float2*>(cp + row * RS + 2 * k) = make_float2(f64_to_f32(v.x), f64_to_f32(v.y));
  }
}

// A site's 24 components from a staged row into registers (16-byte loads).
__device__ __forceinline__ void load_row(const float* __restrict__ p, float r[24]) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    float4 const v = reinterpret_cast<const float4*>(p)[i];
    r[4 * i] = v.x; r[4 * i + 1] = v.y; r[4 * i + 2] = v.z; r[4 * i + 3] = v.w;
  }
}
__device__ __forceinline__ void load_row(const double* __restrict__ p, double r[24]) {
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    double2 const v = reinterpret_cast<const double2*>(p)[i];
    r[2 * i] = v.x; r[2 * i + 1] = v.y;
  }
}


// Pass 1's FP32 path: convert a landed FP64 stage into the FP32 compute copy
// and, in the same pass, into the FP32 tile copies (y32 by pair 0's CTAs).
// One unit = (row, 16-byte group c4, site); consecutive threads take
// consecutive sites, so the global stores of 8 threads cover 128 contiguous
// bytes.
template <int NF, int TS>
__device__ __forceinline__ void convert_and_copy(const double* __restrict__ st, float* __restrict__ cp,
                                                 float* __restrict__ a32, float* __restrict__ b32, int f0,
                                                 long long V, long long s0, int nvalid) {
  static_assert(32 % TS == 0, "a tile lies inside one 32-site tile of the copy");
  constexpr int kRows = 2 * NF * 12, RS = row_stride<float, TS>();
  long long const nt32 = (V + 31) / 32;
  for (int u = threadIdx.x; u < kRows * 6 * TS; u += blockDim.x) {
    int const si = u % TS, c4 = (u / TS) % 6, row = u / (6 * TS);
    if (si >= nvalid) continue;
    const double2* src = reinterpret_cast<const double2*>(st + ((size_t)row * TS + si) * 24 + 4 * c4);
    double2 const v0 = src[0], v1 = src[1];
    float4 const f = make_float4(f64_to_f32(v0.x), f64_to_f32(v0.y), f64_to_f32(v1.x), f64_to_f32(v1.y));
    *reinterpret_cast<float4*>(cp + (size_t)row * RS + si * 24 + 4 * c4) = f;
    int const which = row / (NF * 12), fl = (row / 12) % NF, ia = row % 12;
    float* dst = which == 0 ? a32 : b32;
    if (dst != nullptr) {
      int const ff = which == 0 ? f0 + fl : 1 - f0 - fl;
      long long const v = s0 + si;
      *reinterpret_cast<float4*>(dst + ((size_t)(ff * 12 + ia) * nt32 + (size_t)(v >> 5)) * (32 * 24) +
                                 f32_tile_off((int)(v & 31), c4)) = f;
    }
  }
}

// ---------------------------------------------------------------------------
// Pass 1 (ker_dzu_dzsu, cuda_lattice.cu:160-262), per CTA partial sums.
// Thread (fl, ia, ib) owns dzu[k][ia][ib] and dzsu[s][ia][ib] of flavour
// f = f0 + fl: with A = fwd_src[f][ia](z), B = fwd_y[1-f][ib](z),
//   X_s(z)  = sum_i conj(B_i) (g5 g_s A)_i
//   dzsu[s] += X_s,   dzu[k] += zh_rho(z) X_sigma - zh_sigma(z) X_rho.
// X_s is assembled from the eight spin-block products
//   P[s1][s2] = sum_c conj(B[s1][c]) A[s2][c],  s2 = src(s, s1),
// which is all of g5 g_s's support. Per-site products in T, accumulated per
// tile in T, then into FP64 per tile.
// FP32 path: as it converts a tile, pass 1 also writes it into the FP32
// tile copies the tensor-core pass 2 reads (y32 by pair 0's CTAs, each
// partner's by its own; null pointers: no copy).
template <typename T, int NF, int TS>
__global__ void __launch_bounds__(NF * 144, sizeof(T) == sizeof(float) ? 2 : 1)
p1_kernel(const double* __restrict__ y, PairBatch batch, Geometry geo, int f0,
          double* __restrict__ partials, int* __restrict__ err, float* __restrict__ y32) {
  constexpr int kRows = 2 * NF * 12;
  constexpr size_t kStage = (size_t)kRows * TS * 24;  // doubles per stage
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* s_stage = reinterpret_cast<double*>(smem_raw);         // [2][kRows][TS][24]
  // zerohalf weights of the tile's sites, converted once (a per-thread
  // int -> float conversion issues on GB300's slow FP64/conversion pipe)
  T* s_zh = reinterpret_cast<T*>(smem_raw + stage_bytes<T, NF, TS>());  // [TS][4]
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ int s_fail;

  int const pi = blockIdx.y;
  const double* __restrict__ src = batch.p[pi].src;
  int const gsx[4] = {batch.p[pi].gsx[0], batch.p[pi].gsx[1], batch.p[pi].gsx[2], batch.p[pi].gsx[3]};
  int const t = threadIdx.x;
  int const fl = t / 144, ia = (t % 144) / 12, ib = t % 12;

  // Per-thread sums over this CTA's tiles, each tile's sum added in:
  // compensated FP64 on the FP64 path, compensated FP32 (Kahan) on the FP32
  // path, converted to FP64 at the end.
  constexpr bool kComp = sizeof(T) == sizeof(double);
  using Acc = typename std::conditional<kComp, Neu, KahanF>::type;
  Acc acc_u[6][2], acc_s[4][2];
  T tu[6][2], ts[4][2];
#pragma unroll
  for (int k = 0; k < 6; ++k) tu[k][0] = tu[k][1] = T(0);
#pragma unroll
  for (int s = 0; s < 4; ++s) ts[s][0] = ts[s][1] = T(0);
  auto flush = [&]() {
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        acc_u[k][e].add(tu[k][e]);
        tu[k][e] = T(0);
      }
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        acc_s[s][e].add(ts[s][e]);
        ts[s][e] = T(0);
      }
  };

  constexpr bool kDB = sizeof(T) == sizeof(double);  // double-buffered FP64 stages
  float* s_copy = reinterpret_cast<float*>(s_stage + kStage);  // FP32 mode: the converted tile
  if (t == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
    s_fail = 0;
  }
  __syncthreads();
  long long const ntiles = (geo.V + TS - 1) / TS;
  long long tile = blockIdx.x;
  // src flavour f0+fl, y flavour 1-(f0+fl)
  if (t == 0 && tile < ntiles) issue_tile<NF, TS>(s_stage, &s_bar[0], src, y, f0, 1, 1 - f0, -1, geo.V, tile * TS);
  bool next_in_flight = false;
  int i = 0;
  for (; tile < ntiles; ++i, tile += gridDim.x) {
    int const st = kDB ? (i & 1) : 0;
    long long const s0 = tile * TS;
    int const nvalid = (int)min((long long)TS, geo.V - s0);
    next_in_flight = tile + gridDim.x < ntiles;
    // FP64: prefetch into the other stage (its readers passed the last barrier)
    if (kDB && t == 0 && next_in_flight) {
      fence_proxy_async_smem();
      issue_tile<NF, TS>(s_stage + (st ^ 1) * kStage, &s_bar[st ^ 1], src, y, f0, 1, 1 - f0, -1,
                         geo.V, (tile + gridDim.x) * TS);
    }
    for (int s = t; s < TS; s += blockDim.x) {
      int rel[4];
      rel_coords_fast(geo, gsx, min(s0 + s, geo.V - 1), rel);
#pragma unroll
      for (int r = 0; r < 4; ++r) s_zh[s * 4 + r] = (T)coord_map_zerohalf(rel[r], geo.global[r]);
    }
    uint32_t const parity = kDB ? (uint32_t)((i >> 1) & 1) : (uint32_t)(i & 1);
    if (!mbar_wait(&s_bar[st], parity)) s_fail = 1;
    __syncthreads();
    if (s_fail) break;
    const T* tile_data;
    if constexpr (kDB) {
      tile_data = reinterpret_cast<const T*>(s_stage + st * kStage);
    } else {
      // FP32: convert once, then the stage takes the next tile while we compute
      convert_and_copy<NF, TS>(s_stage, s_copy, batch.p[pi].src32, pi == 0 ? y32 : nullptr, f0, geo.V, s0,
                               nvalid);
      __syncthreads();
      if (t == 0 && next_in_flight) {
        fence_proxy_async_smem();
        issue_tile<NF, TS>(s_stage, &s_bar[0], src, y, f0, 1, 1 - f0, -1, geo.V, (tile + gridDim.x) * TS);
      }
      tile_data = reinterpret_cast<const T*>(s_copy);
    }

    constexpr int RS = row_stride<T, TS>();
    const T* A_base = tile_data + ((size_t)(0 * NF + fl) * 12 + ia) * RS;
    const T* B_base = tile_data + ((size_t)(1 * NF + fl) * 12 + ib) * RS;
#pragma unroll 1
    for (int s = 0; s < nvalid; ++s) {
      // FP32: the site's rows into registers with 16-byte loads; FP64: read
      // in place (two rows of doubles would crowd the registers)
      T Ar[24], Br[24];
      const T* A = A_base + s * 24;
      const T* B = B_base + s * 24;
      if constexpr (sizeof(T) == sizeof(float)) {
        load_row(A, Ar);
        load_row(B, Br);
        A = Ar;
        B = Br;
      }
      // P[s1][s2] for s2 = s1^2 (gamma_0, gamma_3) and s2 = 3-s1 (gamma_1, gamma_2)
      T pa[4][2], pb[4][2];
#pragma unroll
      for (int s1 = 0; s1 < 4; ++s1) {
        T ar = 0, ai = 0, br = 0, bi = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T const yr = (T)B[2 * (3 * s1 + c)], yi = (T)B[2 * (3 * s1 + c) + 1];
          int const sa = s1 ^ 2, sb = 3 - s1;
          T const xr = (T)A[2 * (3 * sa + c)], xi = (T)A[2 * (3 * sa + c) + 1];
          T const zr = (T)A[2 * (3 * sb + c)], zi = (T)A[2 * (3 * sb + c) + 1];
          ar += yr * xr + yi * xi;  ai += yr * xi - yi * xr;
          br += yr * zr + yi * zi;  bi += yr * zi - yi * zr;
        }
        pa[s1][0] = ar; pa[s1][1] = ai; pb[s1][0] = br; pb[s1][1] = bi;
      }
      T X[4][2];
#pragma unroll
      for (int sg = 0; sg < 4; ++sg) {
        T xr = 0, xi = 0;
#pragma unroll
        for (int s1 = 0; s1 < 4; ++s1) {
          T const* pp = (sg == 0 || sg == 3) ? pa[s1] : pb[s1];
          T vr, vi;
          mul_iph(g5g_ph(sg, s1), pp[0], pp[1], vr, vi);
          xr += vr; xi += vi;
        }
        X[sg][0] = xr; X[sg][1] = xi;
      }
      const T* zh = s_zh + s * 4;
#pragma unroll
      for (int sg = 0; sg < 4; ++sg) { ts[sg][0] += X[sg][0]; ts[sg][1] += X[sg][1]; }
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        int const r = comb_rho(k), g = comb_sigma(k);
        T const wr = (T)zh[r], wg = (T)zh[g];
        tu[k][0] += wr * X[g][0] - wg * X[r][0];
        tu[k][1] += wr * X[g][1] - wg * X[r][1];
      }
    }
    flush();
    __syncthreads();
  }
  flush();
  if (s_fail) {
    // a wait gave up: report it, and let no copy into this CTA's shared
    // memory outlive it (bounded, as everything else)
    if (t == 0) {
      if (err) atomicExch(err, kErrWaitTimeout);
      if (kDB && next_in_flight) mbar_wait(&s_bar[(i + 1) & 1], (uint32_t)(((i + 1) >> 1) & 1));
    }
    return;
  }

  double* out = partials + (((size_t)pi * gridDim.x + blockIdx.x) * NF + fl) * kDzLen;
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

// Fixed-order, compensated (Neumaier) FP64 sum over the CTAs' partials.
// dz[fl][i] = sum_cta partials[cta][fl][i]; if add_to != null also
// add_to[fl][i] += dz (the reference's accumulate-into-caller semantics).
// A CTA takes 32 outputs; its 8 warps each sum every 8th CTA's partials
// (compensated), then one warp adds the 8 partial sums in order: 8x the
// warps of one thread per output, each with an eighth of the chain.
constexpr int kRedOut = 32, kRedGrp = 8;
static __global__ void __launch_bounds__(kRedOut * kRedGrp)
    p1_reduce_kernel(const double* __restrict__ partials, int ncta, int nf, double* __restrict__ dz,
                     double* add_dzu, double* add_dzsu) {
  int const fl = blockIdx.y, pi = blockIdx.z;
  int const o = threadIdx.x % kRedOut, grp = threadIdx.x / kRedOut;
  int const i = blockIdx.x * kRedOut + o;
  __shared__ double rs[kRedGrp][kRedOut], rc[kRedGrp][kRedOut];
  partials += (size_t)pi * ncta * nf * kDzLen;
  double s = 0.0, c = 0.0;
  if (i < kDzLen && fl < nf) {
    for (int b = grp; b < ncta; b += kRedGrp) {
      double const v = partials[((size_t)b * nf + fl) * kDzLen + i];
      double const tt = s + v;
      c += fabs(s) >= fabs(v) ? (s - tt) + v : (v - tt) + s;
      s = tt;
    }
  }
  rs[grp][o] = s;
  rc[grp][o] = c;
  __syncthreads();
  if (grp != 0 || i >= kDzLen || fl >= nf) return;
  s = 0.0;
  c = 0.0;
  for (int g = 0; g < kRedGrp; ++g) {
    c += rc[g][o];
    double const v = rs[g][o];
    double const tt = s + v;
    c += fabs(s) >= fabs(v) ? (s - tt) + v : (v - tt) + s;
    s = tt;
  }
  s += c;
  dz += (size_t)pi * nf * kDzLen;
  dz[fl * kDzLen + i] = s;
  if (add_dzu != nullptr) {
    if (i < kDzuLen) add_dzu[fl * kDzuLen + i] += s;
    else add_dzsu[fl * (kDzLen - kDzuLen) + (i - kDzuLen)] += s;
  }
}

// The host gamma insertion of compute_dzu_dzsu (contract.cpp:58-77) on the
// device: g_dzu[k][mu][ia] = g_mu g5 dzu[k][ia], g_dzsu[s][mu][ia] the same.
static __global__ void g_build_kernel(const double* __restrict__ dz, int nf, double* __restrict__ g) {
  int const fl = blockIdx.y, pi = blockIdx.z;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;  // complex index into g
  if (i >= kGLen / 2 || fl >= nf) return;
  dz += (size_t)pi * nf * kDzLen;
  g += (size_t)pi * nf * kGLen;
  // g layout: [j][mu][ia][ib] complex, j < 6 from dzu, else dzsu
  int const ib = i % 12, ia = (i / 12) % 12, mu = (i / 144) % 4, j = i / 576;
  int const sp = ib / 3, cp = ib % 3;
  int const sp2 = gg5_src(mu, sp);
  const double* d = dz + fl * kDzLen + (j < 6 ? 0 : kDzuLen);
  int const jj = j < 6 ? j : j - 6;
  const double* v = d + ((jj * 12 + ia) * 12 + (3 * sp2 + cp)) * 2;
  double re, im;
  mul_iph(gg5_ph(mu, sp), v[0], v[1], re, im);
  g[(size_t)fl * kGLen + 2 * i] = re;
  g[(size_t)fl * kGLen + 2 * i + 1] = im;
}

// Bt[k][n] for pass 2, from g_dzu and g_dzsu (reference layout; flavour fl
// at offset fl*g_stride in both):
//   n = (j*4 + nu)*4 + lambda, M_{j nu lambda} = Gt_lambda B_j Gt_nu with
//   Gt = (g_lambda g5)^T, so M[q][p] = i^ph(lambda, q') g_j[nu][q'][p],
//   q' the spin mapped to q by (g_lambda g5)^T.
//   k = 2*(p*12 + q) + e: Bt = Re M[q][p] (e = 0), -Im M[q][p] (e = 1),
// so that Re Tr(D M) = sum_k Dr[k] Bt[k][n] with Dr = (Re D[p][q], Im D[p][q]).
template <typename T>
__global__ void bt_build_kernel(const double* __restrict__ g_dzu, const double* __restrict__ g_dzsu,
                                size_t g_stride, size_t g_pstride, int nf, T* __restrict__ bt) {
  int const fl = blockIdx.y, pi = blockIdx.z;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kBtK * kBtN || fl >= nf) return;
  g_dzu += (size_t)pi * g_pstride;
  g_dzsu += (size_t)pi * g_pstride;
  bt += (size_t)pi * nf * kBtK * kBtN;
  int const k = i / kBtN, n = i % kBtN;
  int const e = k & 1, pq = k >> 1, p = pq / 12, q = pq % 12;
  int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
  int const sq = q / 3, cq = q % 3;
  int sq2 = 0;
#pragma unroll
  for (int s = 0; s < 4; ++s)
    if (gg5_src(lam, s) == sq) sq2 = s;
  int const ph = gg5_ph(lam, sq2);
  const double* v = j < 6 ? g_dzu + fl * g_stride + ((((j * 4 + nu) * 12) + (3 * sq2 + cq)) * 12 + p) * 2
                          : g_dzsu + fl * g_stride + (((((j - 6) * 4 + nu) * 12) + (3 * sq2 + cq)) * 12 + p) * 2;
  double re, im;
  mul_iph(ph, v[0], v[1], re, im);
  bt[(size_t)fl * kBtK * kBtN + i] = (T)(e == 0 ? re : -im);
}

// ---------------------------------------------------------------------------
// Pass 2 (ker_4pt_contraction, cuda_lattice.cu:277-484), per CTA partials.
// Per site x and flavour f (S = fwd_src[1-f](x), Y = fwd_y[f](x)):
//   D_mu[p][q] = -sum_i conj((g5 g_mu S[q])_i) Y[p]_i                (:323-345)
//   F[mu][n]   = Re Tr(D_mu M_n) = sum_k Dr_mu[k] Bt[k][n]
//   corr_I[k mu nu lam]  = -F[mu][(k, nu, lam)]                       (:346-400)
//   corr_II[k mu nu lam] = -(zh_rho F[mu][(6+sigma,nu,lam)] - zh_sigma F[mu][(6+rho,nu,lam)])
//   dtmp = -sum_{mu,n} coef[mu][n] F[mu][n]                           (:428-476)
// where coef folds the three QED kernels K1 = K(x,y), K2 = K(y,x),
// K3 = K(x, x-y) and the zerohalf weights:
//   coef[mu][(k,nu,lam)]   = K1[k][mu][nu][lam] + K2[k][nu][mu][lam] - K3[k][lam][nu][mu]
//   coef[mu][(6+t,nu,lam)] = sum_k K3[k][lam][nu][mu] (zh_rho_k [sigma_k = t] - zh_sigma_k [rho_k = t]).
// One component kerv[k][mu][nu][lam] of the stand-in QED tensor
// (include/hlbl_gb300_qed.h, hlbl_qed_entry) in the compute type T, from
// q = (a[4], b[4], w[6]): the kernel's two arguments and its six weights.
template <typename T>
__device__ __forceinline__ T qed_entry_t(const T* __restrict__ q, int k, int mu, int nu, int lam) {
  const T* a = q;
  const T* b = q + 4;
  const T* w = q + 8;
  int const r = comb_rho(k), s = comb_sigma(k);
  T v = T(0);
  if (mu == r && nu == s) v += w[0] * a[lam];
  if (mu == s && nu == r) v -= w[0] * a[lam];
  if (mu == r && lam == s) v += w[1] * b[nu];
  if (mu == s && lam == r) v -= w[1] * b[nu];
  if (nu == r && lam == s) v += w[2] * (a[mu] - b[mu]);
  if (nu == s && lam == r) v -= w[2] * (a[mu] - b[mu]);
  if (mu == nu) v += w[3] * (a[r] * b[s] - a[s] * b[r]) * (a[lam] + b[lam]);
  if (mu == s) v += w[4] * a[r] * b[nu] * b[lam];
  if (mu == r) v -= w[4] * a[s] * b[nu] * b[lam];
  if (lam == s) v += w[5] * b[r] * a[mu] * a[nu];
  if (lam == r) v -= w[5] * b[s] * a[mu] * a[nu];
  return v;
}
constexpr int kQ = 14;  // per (site, evaluation): a[4], b[4], w[6]

// four consecutive elements from shared memory (16-byte aligned)
__device__ __forceinline__ void lds4(const float* p, float o[4]) {
  float4 const v = *reinterpret_cast<const float4*>(p);
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void lds4(const double* p, double o[4]) {
  double2 const u = *reinterpret_cast<const double2*>(p);
  double2 const v = *reinterpret_cast<const double2*>(p + 2);
  o[0] = u.x; o[1] = u.y; o[2] = v.x; o[3] = v.y;
}
// CW consecutive elements from global memory (read-only path)
template <int CW>
__device__ __forceinline__ void ldg_cols(const float* p, float o[CW]) {
  if constexpr (CW == 2) {
    float2 const v = __ldg(reinterpret_cast<const float2*>(p));
    o[0] = v.x; o[1] = v.y;
  } else {
#pragma unroll
    for (int c = 0; c < CW; ++c) o[c] = __ldg(p + c);
  }
}
template <int CW>
__device__ __forceinline__ void ldg_cols(const double* p, double o[CW]) {
#pragma unroll
  for (int c = 0; c < CW; ++c) o[c] = __ldg(p + c);
}

// ---------------------------------------------------------------------------
// QED weights: for every local site x the six weight functions of the three
// kernel evaluations of pass 2 (cuda_lattice.cu:435, :448, :461):
//   e = 0: K(xm, ym), e = 1: K(ym, xm), e = 2: K(xm, x - y)
// with xm = coord_map(x - gsx) xunit, ym = coord_map(yv) xunit and x - y the
// minimum image (:403-426). Exact FP64 stand-in quadrature, one thread per
// (site, evaluation). w[(site*3 + e)*6 + j].
struct WArgs {
  PairBatch batch;
  double xunit;
  hlbl_qed_params qp;
};

__device__ __forceinline__ void qed_args(const Geometry& geo, const int gsx[4], const int yv[4],
                                         double xunit, long long site, int e, double a[4],
                                         double b[4]) {
  int rel[4];
  rel_coords(geo, gsx, site, rel);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    double const xm = coord_map(rel[r], geo.global[r]) * xunit;
    double const ym = coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]) * xunit;
    double const xmy = coord_map_diff(rel[r], yv[r], geo.global[r]) * xunit;
    a[r] = e == 1 ? ym : xm;
    b[r] = e == 0 ? ym : (e == 1 ? xm : xmy);
  }
}

static __global__ void qed_weights_exact_kernel(Geometry geo, WArgs args, double* __restrict__ w) {
  long long const n = geo.V * 3;
  int const pi = blockIdx.y;
  int const gsx[4] = {args.batch.p[pi].gsx[0], args.batch.p[pi].gsx[1], args.batch.p[pi].gsx[2], args.batch.p[pi].gsx[3]};
  int const yv[4] = {args.batch.p[pi].yv[0], args.batch.p[pi].yv[1], args.batch.p[pi].yv[2], args.batch.p[pi].yv[3]};
  w += (size_t)pi * n * HLBL_QED_NW;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double a[4], b[4], X, c, Y, ww[HLBL_QED_NW];
    qed_args(geo, gsx, yv, args.xunit, i / 3, (int)(i % 3), a, b);
    hlbl_qed_invariants(a, b, &X, &c, &Y);
    hlbl_qed_weights(&args.qp, X, c, Y, ww);
#pragma unroll
    for (int j = 0; j < HLBL_QED_NW; ++j) w[i * HLBL_QED_NW + j] = ww[j];
  }
}

// The mixed-precision path's exact weight: the same 16-node quadrature in
// FP32 where min(|a|, |b|) >= r64 (every quadrature term is positive, so
// FP32 keeps a few 1e-7 relative accuracy; qed_f32.cuh), in FP64 inside that
// radius (near the origin) -- the FP64 QED evaluation is kept only there.
// One thread per site: its three evaluations share the site's coordinates
// (32-bit integer arithmetic, V < 2^31); the quadrature is FP32; the FP64
// evaluations near the origin are shared by the warp (one node per lane)
// instead of run by single lanes.
static __global__ void qed_weights_fp32_kernel(Geometry geo, WArgs args, double r64, QedF32 qf,
                                               double* __restrict__ w) {
  int const pi = blockIdx.y;
  int const gsx[4] = {args.batch.p[pi].gsx[0], args.batch.p[pi].gsx[1], args.batch.p[pi].gsx[2], args.batch.p[pi].gsx[3]};
  int const yv[4] = {args.batch.p[pi].yv[0], args.batch.p[pi].yv[1], args.batch.p[pi].yv[2], args.batch.p[pi].yv[3]};
  w += (size_t)pi * geo.V * 3 * HLBL_QED_NW;
  unsigned const V = (unsigned)geo.V, stride = gridDim.x * blockDim.x;
  float const xuf = (float)args.xunit, r64f = (float)r64;
  int iy[4], ny = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    iy[r] = coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]);
    ny += iy[r] * iy[r];
  }
  // every lane runs every iteration (the near-origin evaluations are shared
  // by the warp); lanes past the end compute on the last site and store nothing
  for (unsigned base = blockIdx.x * blockDim.x; base < V; base += stride) {
    unsigned const site = min(base + threadIdx.x, V - 1);
    bool const valid = base + threadIdx.x < V;
    unsigned s = site;
    int c[4];
    c[3] = (int)(s % (unsigned)geo.local[3]); s /= (unsigned)geo.local[3];
    c[2] = (int)(s % (unsigned)geo.local[2]); s /= (unsigned)geo.local[2];
    c[1] = (int)(s % (unsigned)geo.local[1]); s /= (unsigned)geo.local[1];
    c[0] = (int)s;
    // the arguments are small integer vectors times xunit: |a|^2, |b|^2 and
    // a.b are exact integer sums (times xunit^2), so |a|, |b| and cos(a, b)
    // come out of correctly rounded FP32 square roots and one division
    // (within 1.5 ulp; the FP64 weight gets the same invariants in FP64)
    int ix[4], ixy[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int const G = geo.global[r];
      int const rel = (c[r] + geo.pc[r] * geo.local[r] - gsx[r] + G) % G;
      ix[r] = coord_map(rel, G);
      ixy[r] = coord_map_diff(rel, yv[r], G);
    }
    int nx = 0, nxy = 0, dxy = 0, dxx = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      nx += ix[r] * ix[r];
      nxy += ixy[r] * ixy[r];
      dxy += ix[r] * iy[r];
      dxx += ix[r] * ixy[r];
    }
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      // e = 0: K(xm, ym), e = 1: K(ym, xm), e = 2: K(xm, x - y)
      int const na = e == 1 ? ny : nx, nb = e == 0 ? ny : (e == 1 ? nx : nxy), nab = e == 2 ? dxx : dxy;
      float const ra = sqrtf((float)na), rb = sqrtf((float)nb);
      float const X = xuf * ra, Y = xuf * rb;
      float cc = (na > 0 && nb > 0) ? (float)nab / (ra * rb) : 0.f;
      cc = fminf(1.f, fmaxf(-1.f, cc));
      bool const near = fminf(X, Y) < r64f;
      double ww[HLBL_QED_NW];
      {
        float wf[HLBL_QED_NW];
        if (qf.geometric) weights_f32<true, false>(qf, X, cc, Y, wf);
        else weights_f32<false, false>(qf, X, cc, Y, wf);
#pragma unroll
        for (int j = 0; j < HLBL_QED_NW; ++j) ww[j] = (double)wf[j];
      }
      double Xd = 0, cd = 0, Yd = 0;
      if (near) {
        Xd = args.xunit * sqrt((double)na);
        Yd = args.xunit * sqrt((double)nb);
        cd = (na > 0 && nb > 0) ? (double)nab / sqrt((double)na * (double)nb) : 0.0;
        cd = cd > 1.0 ? 1.0 : (cd < -1.0 ? -1.0 : cd);
      }
      // near the origin: the FP64 weight of the FP64 arguments, the warp
      // sharing each such evaluation (one quadrature node per lane)
      unsigned const m = __ballot_sync(0xffffffffu, near);
      if (m) qed_weights_fp64_warp(args.qp, m, Xd, cd, Yd, ww);
      if (valid) {
#pragma unroll
        for (int j = 0; j < HLBL_QED_NW; ++j) w[((size_t)site * 3 + e) * HLBL_QED_NW + j] = ww[j];
      }
    }
  }
}

// Coefficient layouts in HBM of the generic QED path (qed_provider.cuh), per
// pair:
//   FP64 (the FP64 pass 2): [V][4][160] doubles, a site's 640 contiguous;
//   FP32 (the tensor-core and CUDA-core FP32 pass 2): tiles of 32 sites,
//     [tile][mu][n/4][32 sites][4] floats, so that the 32 rows (mu, site) of
//     one TMEM lane quadrant read 512 contiguous bytes per group of four n;
//     the last tile is padded with zeros.
constexpr int kCoefPerSite = 4 * kBtN;  // 640
__host__ __device__ __forceinline__ size_t coef32_index(long long site, int mu, int n) {
  long long const tile = site >> 5;
  return ((((size_t)tile * 4 + mu) * (kBtN / 4) + (n >> 2)) * 32 + (size_t)(site & 31)) * 4 + (n & 3);
}
__host__ __device__ __forceinline__ size_t coef32_per_pair(long long V) {
  return (size_t)((V + 31) / 32) * 32 * kCoefPerSite;
}
__host__ __device__ __forceinline__ size_t coef64_per_pair(long long V) {
  return (size_t)V * kCoefPerSite;
}

struct P2Args {
  double xunit;
  int f0;                 // first flavour
  const double* w;        // QED weights [pair][V][3][6] (qed_weights_*_kernel), closed form
  const void* coef;       // or (generic QED path) the coefficients, T of the kernel, in the
                          // FP64 layout for T = double and the FP32 layout for T = float
  size_t coef_stride;     // elements per pair of coef
};

template <typename T, int NF, int TS>
constexpr size_t p2_smem_bytes() {
  return stage_bytes<T, NF, TS>()                      // input staging
         + sizeof(T) * (size_t)(TS * NF * 4 * kBtK     // D
                              + TS * 4 * kBtN)         // coef
         + sizeof(double) * (size_t)(TS * 12)                            // xm, xmy, xvzh
         + sizeof(T) * (size_t)(TS * 3 * kQ);                            // tensor inputs
}

template <typename T, int NF, int TS>
constexpr size_t p1_smem_bytes() {
  return stage_bytes<T, NF, TS>() + sizeof(T) * TS * 4;
}

// The pass-1 variant of hlbl_cu_dzu_dzsu_noalloc: one flavour, FP64, the
// same tile as the context's FP64 pass 1.
struct P1NoAllocTraits {
  static constexpr int kTS = 8;
  static constexpr int kThreads = 144;
  static constexpr size_t kSmem = p1_smem_bytes<double, 1, kTS>();
};

template <typename T, int NF, int TS>
__global__ void __launch_bounds__(NF * 160)
p2_kernel(const double* __restrict__ y, PairBatch batch, Geometry geo, P2Args args,
          const T* __restrict__ bt_all, double* __restrict__ partials, int* __restrict__ err) {
  constexpr int kRows = 2 * NF * 12;
  constexpr size_t kStage = (size_t)kRows * TS * 24;  // doubles per input stage
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* s_stage = reinterpret_cast<double*>(smem_raw);  // FP64 stage(s) (TMA) [+ FP32 copy]
  T* s_D = reinterpret_cast<T*>(smem_raw + stage_bytes<T, NF, TS>());  // [TS][NF][4][288]
  T* s_coef = s_D + TS * NF * 4 * kBtK;          // [TS][4][160]
  double* s_vec = reinterpret_cast<double*>(s_coef + TS * 4 * kBtN);   // [TS][12]
  T* s_q = reinterpret_cast<T*>(s_vec + TS * 12);                      // [TS][3][kQ]

  int const t = threadIdx.x;
  int const nthr = blockDim.x;
  int const pi = blockIdx.y;
  const double* __restrict__ src = batch.p[pi].src;
  int const gsx[4] = {batch.p[pi].gsx[0], batch.p[pi].gsx[1], batch.p[pi].gsx[2], batch.p[pi].gsx[3]};
  int const yv[4] = {batch.p[pi].yv[0], batch.p[pi].yv[1], batch.p[pi].yv[2], batch.p[pi].yv[3]};
  const double* __restrict__ wq = args.w ? args.w + (size_t)pi * geo.V * 3 * HLBL_QED_NW : nullptr;
  const T* __restrict__ bt = bt_all + (size_t)pi * NF * kBtK * kBtN;
  double const xu = args.xunit;
  double ym[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ym[r] = coord_map(mod_pos(yv[r], geo.global[r]), geo.global[r]) * xu;

  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ int s_fail;
  if (t == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
    s_fail = 0;
  }
  __syncthreads();

  Neu run;  // this thread's compensated FP64 running sum for its flavour
  long long const ntiles = (geo.V + TS - 1) / TS;
  long long tile = blockIdx.x;
  constexpr bool kDB = sizeof(T) == sizeof(double);  // double-buffered FP64 stages
  float* s_copy = reinterpret_cast<float*>(s_stage + kStage);  // FP32 mode: the converted tile
  // S = src at flavour 1-f, Y = y at flavour f
  if (t == 0 && tile < ntiles)
    issue_tile<NF, TS>(s_stage, &s_bar[0], src, y, 1 - args.f0, -1, args.f0, 1, geo.V, tile * TS);
  bool next_in_flight = false;
  int it_tile = 0;
  for (; tile < ntiles; ++it_tile, tile += gridDim.x) {
    long long const s0 = tile * TS;
    int const st = kDB ? (it_tile & 1) : 0;
    int const nvalid = (int)min((long long)TS, geo.V - s0);
    // FP64: prefetch the next tile into the other stage while this one is computed
    next_in_flight = tile + gridDim.x < ntiles;
    if (kDB && t == 0 && next_in_flight) {
      fence_proxy_async_smem();
      issue_tile<NF, TS>(s_stage + (st ^ 1) * kStage, &s_bar[st ^ 1], src, y, 1 - args.f0, -1,
                         args.f0, 1, geo.V, (tile + gridDim.x) * TS);
    }
    // per site: xm, x - y (minimum image) and the zerohalf weights
    for (int it = t; it < TS * 4; it += nthr) {
      int const s = it >> 2, r = it & 3;
      int rel[4];
      rel_coords_fast(geo, gsx, min(s0 + s, geo.V - 1), rel);
      s_vec[s * 12 + r] = coord_map(rel[r], geo.global[r]) * xu;
      s_vec[s * 12 + 4 + r] = coord_map_diff(rel[r], yv[r], geo.global[r]) * xu;
      s_vec[s * 12 + 8 + r] = (double)coord_map_zerohalf(rel[r], geo.global[r]);
    }
    __syncthreads();
    if (args.coef) {
      // generic QED path: the coefficients of the tile's sites (zero past the end)
      const T* cg = static_cast<const T*>(args.coef) + (size_t)pi * args.coef_stride;
      for (int it = t; it < TS * kCoefPerSite; it += nthr) {
        int const s = it / kCoefPerSite, mn = it % kCoefPerSite;
        long long const site = s0 + s;
        T v = T(0);
        if (site < geo.V) {
          if constexpr (sizeof(T) == 8) v = __ldg(cg + (size_t)site * kCoefPerSite + mn);
          else v = __ldg(cg + coef32_index(site, mn / kBtN, mn % kBtN));
        }
        s_coef[it] = v;
      }
    } else {
    // the QED tensor's inputs per (site, evaluation), in T:
    // e = 0: K(x, y), e = 1: K(y, x), e = 2: K(x, x - y)
    for (int it = t; it < TS * 3 * kQ; it += nthr) {
      int const se = it / kQ, i = it % kQ, s = se / 3, e = se % 3;
      const double* xm = s_vec + s * 12;
      const double* xmy = xm + 4;
      double v;
      if (i < 4) v = e == 1 ? ym[i] : xm[i];
      else if (i < 8) v = e == 0 ? ym[i - 4] : (e == 1 ? xm[i - 4] : xmy[i - 4]);
      else v = wq[(size_t)(min(s0 + s, geo.V - 1) * 3 + e) * HLBL_QED_NW + (i - 8)];
      s_q[it] = (T)v;
    }
    __syncthreads();
    // coefficients (site-dependent, flavour-independent), in T
    for (int it = t; it < TS * 4 * kBtN; it += nthr) {
      int const s = it / (4 * kBtN), mu = (it / kBtN) % 4, n = it % kBtN;
      int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
      const T* q1 = s_q + (s * 3 + 0) * kQ;
      const T* q2 = q1 + kQ;
      const T* q3 = q2 + kQ;
      T cf;
      if (j < 6) {
        cf = qed_entry_t(q1, j, mu, nu, lam) + qed_entry_t(q2, j, nu, mu, lam) -
             qed_entry_t(q3, j, lam, nu, mu);
      } else {
        const double* zh = s_vec + s * 12 + 8;
        int const tau = j - 6;
        cf = T(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          int const r = comb_rho(k), g = comb_sigma(k);
          if (g == tau) cf += (T)zh[r] * qed_entry_t(q3, k, lam, nu, mu);
          if (r == tau) cf -= (T)zh[g] * qed_entry_t(q3, k, lam, nu, mu);
        }
      }
      s_coef[(s * 4 + mu) * kBtN + n] = (s0 + s < geo.V) ? cf : T(0);
    }
    }
    // the tile's blocks
    uint32_t const parity = kDB ? (uint32_t)((it_tile >> 1) & 1) : (uint32_t)(it_tile & 1);
    if (!mbar_wait(&s_bar[st], parity)) s_fail = 1;
    __syncthreads();
    if (s_fail) break;
    const T* tile_data;
    if constexpr (kDB) {
      tile_data = reinterpret_cast<const T*>(s_stage + st * kStage);
    } else {
      // FP32: convert once, then the stage takes the next tile while we compute
      convert_stage<NF, TS>(s_stage, s_copy);
      __syncthreads();
      if (t == 0 && next_in_flight) {
        fence_proxy_async_smem();
        issue_tile<NF, TS>(s_stage, &s_bar[0], src, y, 1 - args.f0, -1, args.f0, 1, geo.V,
                           (tile + gridDim.x) * TS);
      }
      tile_data = reinterpret_cast<const T*>(s_copy);
    }
    // D_mu[p][q] for every site and flavour (zero past the tile's valid sites)
    for (int it = t; it < TS * NF * 144; it += nthr) {
      int const s = it / (NF * 144), fl = (it / 144) % NF, pq = it % 144, p = pq / 12, q = pq % 12;
      constexpr int RS = row_stride<T, TS>();
      const T* S = tile_data + ((size_t)(0 * NF + fl) * 12 + q) * RS + s * 24;
      const T* Y = tile_data + ((size_t)(1 * NF + fl) * 12 + p) * RS + s * 24;
      if (s >= nvalid) {
        T* Dz = s_D + ((size_t)(s * NF + fl) * 4) * kBtK + 2 * (p * 12 + q);
#pragma unroll
        for (int mu = 0; mu < 4; ++mu) { Dz[mu * kBtK] = T(0); Dz[mu * kBtK + 1] = T(0); }
        continue;
      }
      // O[s1][s2] = sum_c Y[s1][c] conj(S[s2][c]) for s2 = s1^2 and 3-s1
      T oa[4][2], ob[4][2];
#pragma unroll
      for (int s1 = 0; s1 < 4; ++s1) {
        T ar = 0, ai = 0, br = 0, bi = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T const yr = (T)Y[2 * (3 * s1 + c)], yi = (T)Y[2 * (3 * s1 + c) + 1];
          int const sa = s1 ^ 2, sb = 3 - s1;
          T const xr = (T)S[2 * (3 * sa + c)], xi = (T)S[2 * (3 * sa + c) + 1];
          T const zr = (T)S[2 * (3 * sb + c)], zi = (T)S[2 * (3 * sb + c) + 1];
          ar += yr * xr + yi * xi;  ai += yi * xr - yr * xi;
          br += yr * zr + yi * zi;  bi += yi * zr - yr * zi;
        }
        oa[s1][0] = ar; oa[s1][1] = ai; ob[s1][0] = br; ob[s1][1] = bi;
      }
      T* Dout = s_D + ((size_t)(s * NF + fl) * 4) * kBtK + 2 * (p * 12 + q);
#pragma unroll
      for (int mu = 0; mu < 4; ++mu) {
        T dr = 0, di = 0;
#pragma unroll
        for (int s1 = 0; s1 < 4; ++s1) {
          T const* o = (mu == 0 || mu == 3) ? oa[s1] : ob[s1];
          // -conj(i^ph) * O = i^(2 - ph) * O  ... conj(i^ph) = i^(-ph)
          T vr, vi;
          mul_iph((6 - g5g_ph(mu, s1)) & 3, o[0], o[1], vr, vi);
          dr += vr; di += vi;
        }
        Dout[mu * kBtK] = dr;
        Dout[mu * kBtK + 1] = di;
      }
    }
    __syncthreads();
    // F = Dr . Bt and the coefficient dot. Thread (fl, part, column group):
    // CW adjacent columns n for TS/SPLIT sites and the 4 mu, k in steps of 4
    // (128-bit shared loads of D, broadcast across the warp).
    {
      constexpr int CW = sizeof(T) == 4 ? 2 : 1;
      constexpr int SPLIT = sizeof(T) == 4 ? 2 : 1;
      constexpr int TSS = TS / SPLIT;
      constexpr int NCOL = kBtN / CW;
      static_assert(SPLIT * NCOL == kBtN, "one flavour's threads cover its columns once");
      int const fl = t / kBtN, r = t % kBtN;
      int const part = r / NCOL, n0 = (r % NCOL) * CW;
      T acc[TSS][4][CW];
#pragma unroll
      for (int s = 0; s < TSS; ++s)
#pragma unroll
        for (int mu = 0; mu < 4; ++mu)
#pragma unroll
          for (int c = 0; c < CW; ++c) acc[s][mu][c] = T(0);
      const T* B = bt + (size_t)fl * kBtK * kBtN + n0;
      const T* Db = s_D + ((size_t)(part * TSS) * NF + fl) * 4 * kBtK;
#pragma unroll 2
      for (int k = 0; k < kBtK; k += 4) {
        T b[4][CW];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) ldg_cols<CW>(B + (size_t)(k + kk) * kBtN, b[kk]);
#pragma unroll
        for (int s = 0; s < TSS; ++s)
#pragma unroll
          for (int mu = 0; mu < 4; ++mu) {
            T d[4];
            lds4(Db + ((size_t)s * NF * 4 + mu) * kBtK + k, d);
#pragma unroll
            for (int c = 0; c < CW; ++c) {
              // one FMA per product, accumulated in order (no extra add)
              T a = acc[s][mu][c];
              a = fma(d[0], b[0][c], a);
              a = fma(d[1], b[1][c], a);
              a = fma(d[2], b[2][c], a);
              a = fma(d[3], b[3][c], a);
              acc[s][mu][c] = a;
            }
          }
      }
      T part_sum = T(0);
#pragma unroll
      for (int s = 0; s < TSS; ++s)
#pragma unroll
        for (int mu = 0; mu < 4; ++mu)
#pragma unroll
          for (int c = 0; c < CW; ++c)
            part_sum += s_coef[((part * TSS + s) * 4 + mu) * kBtN + n0 + c] * acc[s][mu][c];
      run.add(-(double)part_sum);
    }
    __syncthreads();  // D, coef and this stage are rewritten in the next iterations
  }
  if (s_fail) {
    if (t == 0) {
      if (err) atomicExch(err, kErrWaitTimeout);
      if (kDB && next_in_flight) mbar_wait(&s_bar[(it_tile + 1) & 1], (uint32_t)(((it_tile + 1) >> 1) & 1));
    }
    return;
  }

  // block reduction per flavour in a fixed order: warp shuffles, then warps
  // (a compensated tree: each level adds the pair's sums and their
  // rounding errors; the error terms travel with them)
  __shared__ double s_red[32][2];
  Neu v = run;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double const os = __shfl_down_sync(0xffffffffu, v.s, o);
    double const oc = __shfl_down_sync(0xffffffffu, v.c, o);
    v.add(os);
    v.c += oc;
  }
  __syncthreads();
  if ((t & 31) == 0) { s_red[t >> 5][0] = v.s; s_red[t >> 5][1] = v.c; }
  __syncthreads();
  if (t < NF) {
    // warps [fl*160/32, (fl+1)*160/32) hold flavour fl (160 = 5 warps)
    Neu s;
    for (int w = t * (kBtN / 32); w < (t + 1) * (kBtN / 32); ++w) { s.add(s_red[w][0]); s.c += s_red[w][1]; }
    partials[((size_t)pi * gridDim.x + blockIdx.x) * NF + t] = s.get();
  }
}

// out[fl] = sum_cta partials[cta][fl] (fixed order, compensated); if add
// is set, out[fl] is added to rather than written.
// One warp per flavour: lane l sums every 32nd CTA's partial (compensated),
// lane 0 adds the 32 lane sums in order (fixed order, deterministic).
static __global__ void __launch_bounds__(64) p2_reduce_kernel(const double* __restrict__ partials, int ncta,
                                                              int nf, PairBatch batch, int add) {
  int const fl = threadIdx.x >> 5, lane = threadIdx.x & 31, pi = blockIdx.x;
  __shared__ double rs[2][32], rc[2][32];
  if (fl >= nf) return;
  partials += (size_t)pi * ncta * nf;
  double s = 0.0, c = 0.0;
  for (int b = lane; b < ncta; b += 32) {
    double const v = partials[(size_t)b * nf + fl];
    double const tt = s + v;
    c += fabs(s) >= fabs(v) ? (s - tt) + v : (v - tt) + s;
    s = tt;
  }
  rs[fl][lane] = s;
  rc[fl][lane] = c;
  __syncwarp();
  if (lane != 0) return;
  s = 0.0;
  c = 0.0;
  for (int l = 0; l < 32; ++l) {
    c += rc[fl][l];
    double const v = rs[fl][l];
    double const tt = s + v;
    c += fabs(s) >= fabs(v) ? (s - tt) + v : (v - tt) + s;
    s = tt;
  }
  s += c;
  double* __restrict__ out = batch.p[pi].out;
  if (add) out[fl] += s;
  else out[fl] = s;
}

}  // namespace hg
