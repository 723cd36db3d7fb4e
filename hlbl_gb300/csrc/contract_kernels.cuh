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

#include "hlbl_device.cuh"

namespace hg {

constexpr int kDzLen = 2880;       // dzu[6][12][12][2] + dzsu[4][12][12][2]
constexpr int kDzuLen = 1728;
constexpr int kGLen = 11520;       // g_dzu[6][4][12][24] + g_dzsu[4][4][12][24]
constexpr int kGDzuLen = 6912;
constexpr int kBtK = 288;          // rows of Bt: (p, q, re/im)
constexpr int kBtN = 160;          // columns of Bt: (j, nu, lambda), j < 10

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

// ---------------------------------------------------------------------------
// Tile loader: rows (which, fl, ia) of the two blocks into shared memory as T.
// which = 0 reads `a` at flavour fa(fl), which = 1 reads `b` at fb(fl).
// Sites past V are zero-filled, so they contribute nothing.
template <typename T, int NF, int TS>
__device__ __forceinline__ void load_tile(T* __restrict__ s_in, const double* __restrict__ a,
                                          const double* __restrict__ b, int fa0, int fa_step,
                                          int fb0, int fb_step, long long V, long long s0) {
  constexpr int kRows = 2 * NF * 12;
  constexpr int kPer = TS * 12;  // double2 per row
  int const nvalid = (int)min((long long)TS, V - s0);
  for (int idx = threadIdx.x; idx < kRows * kPer; idx += blockDim.x) {
    int const row = idx / kPer, w = idx - row * kPer;
    int const which = row / (NF * 12);
    int const fl = (row / 12) % NF;
    int const ia = row % 12;
    int const site = w / 12;
    double2 v = make_double2(0.0, 0.0);
    if (site < nvalid) {
      int const f = which == 0 ? fa0 + fa_step * fl : fb0 + fb_step * fl;
      const double* base = (which == 0 ? a : b) + ((size_t)(f * 12 + ia) * V + s0) * 24;
      v = __ldg(reinterpret_cast<const double2*>(base) + w);
    }
    T* o = s_in + (size_t)row * TS * 24 + 2 * w;
    o[0] = (T)v.x;
    o[1] = (T)v.y;
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
template <typename T, int NF, int TS>
__global__ void __launch_bounds__(NF * 144)
p1_kernel(const double* __restrict__ src, const double* __restrict__ y, Geometry geo,
          int4 gsx4, int f0, double* __restrict__ partials) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_in = reinterpret_cast<T*>(smem_raw);                       // [2][NF][12][TS][24]
  int* s_zh = reinterpret_cast<int*>(s_in + 2 * NF * 12 * TS * 24);  // [TS][4]

  int const gsx[4] = {gsx4.x, gsx4.y, gsx4.z, gsx4.w};
  int const t = threadIdx.x;
  int const fl = t / 144, ia = (t % 144) / 12, ib = t % 12;

  // FP64 per-thread sums over this CTA's tiles: compensated on the FP64
  // path, plain on the FP32 path (whose tile sums are only FP32-accurate).
  constexpr bool kComp = sizeof(T) == sizeof(double);
  Neu acc_u[6][2], acc_s[4][2];

  long long const ntiles = (geo.V + TS - 1) / TS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    long long const s0 = tile * TS;
    __syncthreads();
    // src flavour f0+fl, y flavour 1-(f0+fl)
    load_tile<T, NF, TS>(s_in, src, y, f0, 1, 1 - f0, -1, geo.V, s0);
    for (int s = threadIdx.x; s < TS; s += blockDim.x) {
      int rel[4];
      rel_coords(geo, gsx, min(s0 + s, geo.V - 1), rel);
      bool const ok = s0 + s < geo.V;
#pragma unroll
      for (int r = 0; r < 4; ++r) s_zh[s * 4 + r] = ok ? coord_map_zerohalf(rel[r], geo.global[r]) : 0;
    }
    __syncthreads();

    T tu[6][2], ts[4][2];
#pragma unroll
    for (int k = 0; k < 6; ++k) tu[k][0] = tu[k][1] = T(0);
#pragma unroll
    for (int s = 0; s < 4; ++s) ts[s][0] = ts[s][1] = T(0);

    const T* A_base = s_in + ((size_t)(0 * NF + fl) * 12 + ia) * TS * 24;
    const T* B_base = s_in + ((size_t)(1 * NF + fl) * 12 + ib) * TS * 24;
#pragma unroll 1
    for (int s = 0; s < TS; ++s) {
      const T* A = A_base + s * 24;
      const T* B = B_base + s * 24;
      // P[s1][s2] for s2 = s1^2 (gamma_0, gamma_3) and s2 = 3-s1 (gamma_1, gamma_2)
      T pa[4][2], pb[4][2];
#pragma unroll
      for (int s1 = 0; s1 < 4; ++s1) {
        T ar = 0, ai = 0, br = 0, bi = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T const yr = B[2 * (3 * s1 + c)], yi = B[2 * (3 * s1 + c) + 1];
          int const sa = s1 ^ 2, sb = 3 - s1;
          T const xr = A[2 * (3 * sa + c)], xi = A[2 * (3 * sa + c) + 1];
          T const zr = A[2 * (3 * sb + c)], zi = A[2 * (3 * sb + c) + 1];
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
          T const* p = (sg == 0 || sg == 3) ? pa[s1] : pb[s1];
          T vr, vi;
          mul_iph(g5g_ph(sg, s1), p[0], p[1], vr, vi);
          xr += vr; xi += vi;
        }
        X[sg][0] = xr; X[sg][1] = xi;
      }
      const int* zh = s_zh + s * 4;
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
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        if (kComp) acc_u[k][e].add((double)tu[k][e]);
        else acc_u[k][e].s += (double)tu[k][e];
      }
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        if (kComp) acc_s[s][e].add((double)ts[s][e]);
        else acc_s[s][e].s += (double)ts[s][e];
      }
  }

  double* out = partials + ((size_t)blockIdx.x * NF + fl) * kDzLen;
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
static __global__ void p1_reduce_kernel(const double* __restrict__ partials, int ncta, int nf,
                                 double* __restrict__ dz, double* add_dzu, double* add_dzsu) {
  int const fl = blockIdx.y;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kDzLen || fl >= nf) return;
  double s = 0.0, c = 0.0;
  for (int b = 0; b < ncta; ++b) {
    double const v = partials[((size_t)b * nf + fl) * kDzLen + i];
    double const tt = s + v;
    c += fabs(s) >= fabs(v) ? (s - tt) + v : (v - tt) + s;
    s = tt;
  }
  s += c;
  dz[fl * kDzLen + i] = s;
  if (add_dzu != nullptr) {
    if (i < kDzuLen) add_dzu[fl * kDzuLen + i] += s;
    else add_dzsu[fl * (kDzLen - kDzuLen) + (i - kDzuLen)] += s;
  }
}

// The host gamma insertion of compute_dzu_dzsu (contract.cpp:58-77) on the
// device: g_dzu[k][mu][ia] = g_mu g5 dzu[k][ia], g_dzsu[s][mu][ia] the same.
static __global__ void g_build_kernel(const double* __restrict__ dz, int nf, double* __restrict__ g) {
  int const fl = blockIdx.y;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;  // complex index into g
  if (i >= kGLen / 2 || fl >= nf) return;
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
                                size_t g_stride, int nf, T* __restrict__ bt) {
  int const fl = blockIdx.y;
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kBtK * kBtN || fl >= nf) return;
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
struct P2Args {
  int gsx[4];
  int yv[4];
  double xunit;
  int f0;      // first flavour
  hlbl_qed_params qp;
};

template <typename T, int NF, int TS>
constexpr size_t p2_smem_bytes() {
  return sizeof(T) * (size_t)(2 * NF * 12 * TS * 24     // inputs
                              + TS * NF * 4 * kBtK     // D
                              + TS * 4 * kBtN)         // coef
         + sizeof(double) * (size_t)(TS * 3 * HLBL_QED_NQ * HLBL_QED_NW  // node terms
                                     + TS * 3 * HLBL_QED_NW              // weights
                                     + TS * 12);                         // xm, xmy, xvzh
}

template <typename T, int NF, int TS>
constexpr size_t p1_smem_bytes() {
  return sizeof(T) * (size_t)(2 * NF * 12 * TS * 24) + sizeof(int) * TS * 4;
}

// The pass-1 variant of hlbl_cu_dzu_dzsu_noalloc: one flavour, FP64, the
// same tile as the context's FP64 pass 1.
struct P1NoAllocTraits {
  static constexpr int kTS = 16;
  static constexpr int kThreads = 144;
  static constexpr size_t kSmem = p1_smem_bytes<double, 1, kTS>();
};

template <typename T, int NF, int TS>
__global__ void __launch_bounds__(NF * 160)
p2_kernel(const double* __restrict__ src, const double* __restrict__ y, Geometry geo,
          P2Args args, const T* __restrict__ bt, double* __restrict__ partials) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_in = reinterpret_cast<T*>(smem_raw);
  T* s_D = s_in + 2 * NF * 12 * TS * 24;         // [TS][NF][4][288]
  T* s_coef = s_D + TS * NF * 4 * kBtK;          // [TS][4][160]
  double* s_node = reinterpret_cast<double*>(s_coef + TS * 4 * kBtN);  // [TS][3][NQ][NW]
  double* s_w = s_node + TS * 3 * HLBL_QED_NQ * HLBL_QED_NW;           // [TS][3][NW]
  double* s_vec = s_w + TS * 3 * HLBL_QED_NW;                          // [TS][12]

  int const t = threadIdx.x;
  int const nthr = blockDim.x;
  double const xu = args.xunit;
  double ym[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ym[r] = coord_map(mod_pos(args.yv[r], geo.global[r]), geo.global[r]) * xu;

  Neu run;  // this thread's compensated FP64 running sum for its flavour
  long long const ntiles = (geo.V + TS - 1) / TS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    long long const s0 = tile * TS;
    __syncthreads();
    // S = src at flavour 1-f, Y = y at flavour f
    load_tile<T, NF, TS>(s_in, src, y, 1 - args.f0, -1, args.f0, 1, geo.V, s0);
    // QED kernel: node terms of the three evaluations per site
    for (int it = t; it < TS * 3 * HLBL_QED_NQ; it += nthr) {
      int const s = it / (3 * HLBL_QED_NQ), e = (it / HLBL_QED_NQ) % 3, i = it % HLBL_QED_NQ;
      int rel[4];
      rel_coords(geo, args.gsx, min(s0 + s, geo.V - 1), rel);
      double xm[4], xmy[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        xm[r] = coord_map(rel[r], geo.global[r]) * xu;
        xmy[r] = coord_map_diff(rel[r], args.yv[r], geo.global[r]) * xu;
      }
      if (e == 0 && i == 0) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          s_vec[s * 12 + r] = xm[r];
          s_vec[s * 12 + 4 + r] = xmy[r];
          s_vec[s * 12 + 8 + r] = (double)coord_map_zerohalf(rel[r], geo.global[r]);
        }
      }
      const double* a = e == 1 ? ym : xm;
      const double* b = e == 0 ? ym : (e == 1 ? xm : xmy);
      double X, c, Y;
      hlbl_qed_invariants(a, b, &X, &c, &Y);
      double const u = args.qp.node[i], v = 1.0 - u;
      double r2 = u * u * X * X + v * v * Y * Y - 2.0 * u * v * X * Y * c;
      r2 = r2 > 0 ? r2 : 0.0;
      double const g = args.qp.weight[i] / (1.0 + r2);
      double const rr = sqrt(r2 + args.qp.lambda * args.qp.lambda);
      double const h[HLBL_QED_NW] = {1.0, u, v, u * v, u * u, v * v};
      double* o = s_node + ((s * 3 + e) * HLBL_QED_NQ + i) * HLBL_QED_NW;
#pragma unroll
      for (int j = 0; j < HLBL_QED_NW; ++j) o[j] = g * h[j] * exp(-args.qp.mass[j] * rr);
    }
    __syncthreads();
    for (int it = t; it < TS * 3 * HLBL_QED_NW; it += nthr) {
      int const s = it / (3 * HLBL_QED_NW), e = (it / HLBL_QED_NW) % 3, j = it % HLBL_QED_NW;
      double acc = 0.0;
      for (int i = 0; i < HLBL_QED_NQ; ++i) acc += s_node[((s * 3 + e) * HLBL_QED_NQ + i) * HLBL_QED_NW + j];
      s_w[(s * 3 + e) * HLBL_QED_NW + j] = acc;
    }
    __syncthreads();
    // coefficients (site-dependent, flavour-independent)
    for (int it = t; it < TS * 4 * kBtN; it += nthr) {
      int const s = it / (4 * kBtN), mu = (it / kBtN) % 4, n = it % kBtN;
      int const lam = n & 3, nu = (n >> 2) & 3, j = n >> 4;
      const double* xm = s_vec + s * 12;
      const double* xmy = xm + 4;
      const double* zh = xm + 8;
      const double* w1 = s_w + (s * 3 + 0) * HLBL_QED_NW;
      const double* w2 = s_w + (s * 3 + 1) * HLBL_QED_NW;
      const double* w3 = s_w + (s * 3 + 2) * HLBL_QED_NW;
      double cf;
      if (j < 6) {
        cf = hlbl_qed_entry(w1, xm, ym, j, mu, nu, lam) + hlbl_qed_entry(w2, ym, xm, j, nu, mu, lam) -
             hlbl_qed_entry(w3, xm, xmy, j, lam, nu, mu);
      } else {
        int const tau = j - 6;
        cf = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          int const r = comb_rho(k), g = comb_sigma(k);
          double const wgt = (g == tau ? zh[r] : 0.0) - (r == tau ? zh[g] : 0.0);
          if (wgt != 0.0) cf += wgt * hlbl_qed_entry(w3, xm, xmy, k, lam, nu, mu);
        }
      }
      s_coef[(s * 4 + mu) * kBtN + n] = (s0 + s < geo.V) ? (T)cf : T(0);
    }
    // D_mu[p][q] for every site and flavour
    for (int it = t; it < TS * NF * 144; it += nthr) {
      int const s = it / (NF * 144), fl = (it / 144) % NF, pq = it % 144, p = pq / 12, q = pq % 12;
      const T* S = s_in + ((size_t)(0 * NF + fl) * 12 + q) * TS * 24 + s * 24;
      const T* Y = s_in + ((size_t)(1 * NF + fl) * 12 + p) * TS * 24 + s * 24;
      // O[s1][s2] = sum_c Y[s1][c] conj(S[s2][c]) for s2 = s1^2 and 3-s1
      T oa[4][2], ob[4][2];
#pragma unroll
      for (int s1 = 0; s1 < 4; ++s1) {
        T ar = 0, ai = 0, br = 0, bi = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T const yr = Y[2 * (3 * s1 + c)], yi = Y[2 * (3 * s1 + c) + 1];
          int const sa = s1 ^ 2, sb = 3 - s1;
          T const xr = S[2 * (3 * sa + c)], xi = S[2 * (3 * sa + c) + 1];
          T const zr = S[2 * (3 * sb + c)], zi = S[2 * (3 * sb + c) + 1];
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
    // F = Dr . Bt and the coefficient dot, thread (fl, n)
    if (t < NF * kBtN) {
      int const fl = t / kBtN, n = t % kBtN;
      T acc[TS][4];
#pragma unroll
      for (int s = 0; s < TS; ++s)
#pragma unroll
        for (int mu = 0; mu < 4; ++mu) acc[s][mu] = T(0);
      const T* B = bt + (size_t)fl * kBtK * kBtN + n;
      const T* Db = s_D + (size_t)fl * 4 * kBtK;
#pragma unroll 4
      for (int k = 0; k < kBtK; ++k) {
        T const b = __ldg(B + (size_t)k * kBtN);
#pragma unroll
        for (int s = 0; s < TS; ++s)
#pragma unroll
          for (int mu = 0; mu < 4; ++mu) acc[s][mu] += Db[((size_t)s * NF * 4 + mu) * kBtK + k] * b;
      }
      T part = T(0);
#pragma unroll
      for (int s = 0; s < TS; ++s)
#pragma unroll
        for (int mu = 0; mu < 4; ++mu) part += s_coef[(s * 4 + mu) * kBtN + n] * acc[s][mu];
      run.add(-(double)part);
    }
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
    partials[(size_t)blockIdx.x * NF + t] = s.get();
  }
}

// out[fl] = sum_cta partials[cta][fl] (fixed order, compensated); if add
// is set, out[fl] is added to rather than written.
static __global__ void p2_reduce_kernel(const double* __restrict__ partials, int ncta, int nf,
                                 double* __restrict__ out, int add) {
  int const fl = threadIdx.x;
  if (fl >= nf) return;
  double s = 0.0, c = 0.0;
  for (int b = 0; b < ncta; ++b) {
    double const v = partials[(size_t)b * nf + fl];
    double const tt = s + v;
    c += fabs(s) >= fabs(v) ? (s - tt) + v : (v - tt) + s;
    s = tt;
  }
  s += c;
  if (add) out[fl] += s;
  else out[fl] = s;
}

}  // namespace hg
