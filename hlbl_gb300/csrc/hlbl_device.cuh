// hlbl_device.cuh -- device-side building blocks shared by the kernels:
// gamma matrices of the cvc basis as monomial spin matrices, the lattice
// coordinate rules, and the kernel-parameter structs.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "hlbl_gb300_qed.h"

namespace hg {

// ---- gamma matrices -----------------------------------------------------
// The cvc basis of the reference (src/gamma.cpp:7-45, cuda_lattice.cu:16-51)
// acts on a spinor v[spin][colour] as (gamma_g v)[s] = i^ph(g,s) v[src(g,s)]:
// every row has a single entry, a power of i. g = 0..3 and 5 (4 is unused).
// The two tables below restate the reference's permutation/sign tables in
// that form; tests check them against the reference's apply_gamma.
__host__ __device__ constexpr int gam_src(int g, int s) {
  // gamma_0, gamma_3: spins 0<->2, 1<->3; gamma_1, gamma_2: 0<->3, 1<->2
  return (g == 0 || g == 3) ? (s ^ 2) : ((g == 1 || g == 2) ? (3 - s) : s);
}
__host__ __device__ constexpr int gam_ph(int g, int s) {
  // powers of i: g0 {2,2,2,2} g1 {3,3,1,1} g2 {2,0,0,2} g3 {3,1,1,3} g5 {0,0,2,2}
  return g == 0 ? 2
       : g == 1 ? (s < 2 ? 3 : 1)
       : g == 2 ? ((s == 0 || s == 3) ? 2 : 0)
       : g == 3 ? ((s == 0 || s == 3) ? 3 : 1)
       : g == 5 ? (s < 2 ? 0 : 2)
       : 0;
}
// gamma_5 gamma_mu: (g5 g_mu v)[s] = i^(ph_mu(s) + ph_5(s)) v[src_mu(s)]
__host__ __device__ constexpr int g5g_src(int mu, int s) { return gam_src(mu, s); }
__host__ __device__ constexpr int g5g_ph(int mu, int s) { return (gam_ph(mu, s) + gam_ph(5, s)) & 3; }
// gamma_mu gamma_5: (g_mu g5 v)[s] = i^(ph_mu(s) + ph_5(src_mu(s))) v[src_mu(s)]
__host__ __device__ constexpr int gg5_src(int mu, int s) { return gam_src(mu, s); }
__host__ __device__ constexpr int gg5_ph(int mu, int s) {
  return (gam_ph(mu, s) + gam_ph(5, gam_src(mu, s))) & 3;
}

// z * i^ph
template <typename T>
__host__ __device__ __forceinline__ void mul_iph(int ph, T re, T im, T& ore, T& oim) {
  switch (ph & 3) {
    case 0: ore = re;  oim = im;  break;
    case 1: ore = -im; oim = re;  break;
    case 2: ore = -re; oim = -im; break;
    default: ore = im; oim = -re; break;
  }
}

// ---- coordinate rules (cuda_lattice.cu:128-154) -------------------------
// [-L/2, L/2) with L/2 -> -L/2: every QED kernel argument
__host__ __device__ __forceinline__ int coord_map(int xi, int L) { return xi >= L / 2 ? xi - L : xi; }
// L/2 -> 0: the odd coordinate weights z_rho, x_rho only
__host__ __device__ __forceinline__ int coord_map_zerohalf(int xi, int L) {
  return xi > L / 2 ? xi - L : (xi < L / 2 ? xi : 0);
}
__host__ __device__ __forceinline__ int mod_pos(int a, int L) {
  int const r = a % L;
  return r < 0 ? r + L : r;
}
// minimum-image difference a - b
__host__ __device__ __forceinline__ int coord_map_diff(int a, int b, int L) {
  return coord_map(mod_pos(a - b, L), L);
}

// ---- geometry passed to every kernel ------------------------------------
struct Geometry {
  int local[4];   // T, LX, LY, LZ of this rank's sub-lattice
  int global[4];  // of the whole lattice
  int pc[4];      // this rank's process-grid coordinates
  long long V;    // local volume
};

// Position relative to the source x = gsx of local site `site`, folded
// into [0, L) per direction (cuda_lattice.cu:196-201, 315-318).
__device__ __forceinline__ void rel_coords(const Geometry& g, const int gsx[4], long long site,
                                           int rel[4]) {
  long long s = site;
  int c[4];
  c[3] = (int)(s % g.local[3]); s /= g.local[3];
  c[2] = (int)(s % g.local[2]); s /= g.local[2];
  c[1] = (int)(s % g.local[1]); s /= g.local[1];
  c[0] = (int)s;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int const v = c[r] + g.pc[r] * g.local[r] - gsx[r];
    rel[r] = (v + g.global[r]) % g.global[r];
  }
}

// The same with 32-bit divisions (a handful of instructions each instead of a
// 64-bit division's few dozen) where the volume allows it.
__device__ __forceinline__ void rel_coords_fast(const Geometry& g, const int gsx[4], long long site, int rel[4]) {
  if (g.V > 0xFFFFFFFFLL) {
    rel_coords(g, gsx, site, rel);
    return;
  }
  unsigned s = (unsigned)site;
  int c[4];
  c[3] = (int)(s % (unsigned)g.local[3]); s /= (unsigned)g.local[3];
  c[2] = (int)(s % (unsigned)g.local[2]); s /= (unsigned)g.local[2];
  c[1] = (int)(s % (unsigned)g.local[1]); s /= (unsigned)g.local[1];
  c[0] = (int)s;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int const v = c[r] + g.pc[r] * g.local[r] - gsx[r];
    rel[r] = (v + g.global[r]) % g.global[r];
  }
}

// ---- TMA bulk copies and mbarriers ----------------------------------------
// Tiles of propagator rows are staged with cp.async.bulk (1-D TMA): one
// thread issues a copy per contiguous row run and the mbarrier's transaction
// count tracks the bytes. Every wait is bounded: after kWaitLimit polls the
// waiter gives up and the kernel reports kErrWaitTimeout through its error
// flag instead of spinning forever.
constexpr uint32_t kWaitLimit = 1u << 20;
constexpr int kErrWaitTimeout = 1;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// order this thread's (and, after a barrier, the CTA's) generic-proxy shared
// memory accesses before later async-proxy (TMA) writes to the same bytes
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// FP64 -> FP32, rounded to nearest even, on the integer pipe only (the
// conversion instruction issues on GB300's FP64 pipe, 1/64 of the FP32
// rate). Normal range: the exponent rebased, the top 23 of the 52 mantissa
// bits, plus the increment the 29 dropped bits call for (a carry may run into
// the exponent, as rounding requires; past the largest float it gives inf).
// Outside it, also in integers: FP32 subnormals and zero (the 53-bit
// significand shifted right with the same rounding), overflow to inf, inf and
// NaN kept.
__device__ __forceinline__ float f64_to_f32(double d) {
  unsigned long long const b = (unsigned long long)__double_as_longlong(d);
  uint32_t const hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  uint32_t const sign = hi & 0x80000000u;
  uint32_t const e = (hi >> 20) & 0x7FFu;
  if (e - 897u <= 253u) {
    uint32_t r = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    uint32_t const rest = lo & 0x1FFFFFFFu;
    r += (uint32_t)(rest > 0x10000000u) | ((uint32_t)(rest == 0x10000000u) & (r & 1u));
    return __uint_as_float(sign | r);
  }
  uint32_t r;
  if (e == 0x7FFu) {
    r = ((hi & 0xFFFFFu) | lo) ? 0x7FC00000u : 0x7F800000u;  // NaN (quiet) or inf
  } else if (e > 1150u) {
    r = 0x7F800000u;  // beyond the float range: inf
  } else if (e < 873u) {
    r = 0u;           // below half the smallest subnormal: zero
  } else {
    // |d| = m * 2^(e - 1075), m the 53-bit significand (e = 0 has none: too
    // small to matter here); in units of 2^-149: m >> (926 - e), 30..53 bits
    unsigned long long const m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    uint32_t const sh = 926u - e;
    unsigned long long const q = m >> sh, rest = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    r = (uint32_t)q + (uint32_t)(rest > half || (rest == half && (q & 1ull)));
  }
  return __uint_as_float(sign | r);
}

// An FP32 tile copy of a block: rows (f, ia) of tiles of 32 sites, a tile's
// row = [half of the tile][16-byte group c4][site in the half][4] floats, so
// that a half tile (16 sites) of a row is 1.5 KB contiguous and a tile 3 KB.
// Offset of (site s of its tile, group c4) within a tile's row:
__host__ __device__ constexpr int f32_tile_off(int s, int c4) { return (s >> 4) * 384 + c4 * 64 + (s & 15) * 4; }

// Kahan's compensated FP32 sum (s - c is the sum): the FP32 path's per-thread
// sums over its tiles, kept off GB300's FP64 pipe (1/64 of the FP32 rate)
// until the end.
struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float const y = v - c;
    float const t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

// (rho, sigma) of the six pairs k, cuda_lattice.cu:52-60
__host__ __device__ constexpr int comb_rho(int k) { return k < 3 ? 0 : (k < 5 ? 1 : 2); }
__host__ __device__ constexpr int comb_sigma(int k) { return k < 3 ? k + 1 : (k < 5 ? k - 1 : 3); }

}  // namespace hg
