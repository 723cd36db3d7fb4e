/*
 * hlbl_gb300.h -- C ABI of the GB300 connected-HLbL contraction library
 * (libhlbl_gb300.so). Plain pointers and sizes only.
 *
 * Device pointers are CUDA device addresses on the context's device. A
 * propagator block is [2 flavours][12 source spin-colour][V sites][24
 * doubles] (src/provider.cpp:45; provider.hpp:18-20), 16-byte aligned, with
 * sites in tmLQCD order ((t*LX + x)*LY + y)*LZ + z (lattice.hpp:32-34).
 * Coordinates are (t, x, y, z); `gsx` is the global site of the source x in
 * [0, L); `yv` is y - x (any integers; the kernels fold it as the reference
 * does).
 *
 * Every function returns 0 on success and a nonzero HLBL_E* code on failure;
 * hlbl_last_error() then describes the failure (thread-local). Functions
 * that take a context run on its stream (hlbl_ctx_set_stream).
 */
#ifndef HLBL_GB300_H
#define HLBL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  HLBL_OK = 0,
  HLBL_EINVAL = 1,   /* bad argument: null, misaligned, out of range */
  HLBL_ECUDA = 2,    /* a CUDA runtime call failed */
  HLBL_ESTATE = 3,   /* call not valid in the context's state */
  HLBL_ENOMEM = 4    /* an allocation failed */
};

/* Precision of the per-site spin-colour products. */
enum { HLBL_FP64 = 0, HLBL_FP32 = 1 };
/* QED weight: the exact FP64 stand-in, or the learned surrogate. */
enum { HLBL_QED_EXACT = 0, HLBL_QED_SURROGATE = 1 };

typedef struct hlbl_ctx hlbl_ctx;

/* Message of the last failed call on this thread ("" if none). */
const char* hlbl_last_error(void);
/* Library version string. */
const char* hlbl_version(void);

/* A contraction context: the lattice (global extents, this rank's local
 * extents and process-grid coordinates), the QED kernel's Lambda, and the
 * device. Owns its work buffers and a stream. Replaces the construction of
 * hlbl::Contractor (include/hlbl/contract.hpp:44, src/contract.cpp:28-31)
 * and KQED's initialise() (bin/hlbl_hypercube.cpp:174-178). */
int hlbl_ctx_create(hlbl_ctx** out, const int global[4], const int local[4],
                    const int proc_coords[4], double lambda, int device);
void hlbl_ctx_destroy(hlbl_ctx* ctx);
/* Waits for the context's stream and reports HLBL_ECUDA if a contraction
 * kernel gave up a bounded wait for a staged tile since the last check (the
 * sums computed since then are invalid); clears the flag. hlbl_kernel_sum
 * checks by itself. */
int hlbl_ctx_check(hlbl_ctx* ctx);
/* Diagnostic of that path: a kernel whose wait can never complete gives up
 * after its bounded wait (about a second), sets the flag and returns; the
 * next hlbl_ctx_check reports it. Nothing faults and the context stays
 * usable. */
int hlbl_selftest_wait_timeout(hlbl_ctx* ctx);
/* Run on `stream` (a cudaStream_t) from now on; NULL restores the context's
 * own stream. */
int hlbl_ctx_set_stream(hlbl_ctx* ctx, void* stream);

/* The kernel sum of both flavours for the pair (x = gsx, y = gsx + yv):
 * out[f] = sum over this rank's sites. Blocking: returns after the result is
 * on the host. Replaces Contractor::kernel_sum (src/contract.cpp:104-114;
 * include/hlbl/contract.hpp:47-49), which also all-reduces over ranks; with
 * more than one rank the caller sums out[] over ranks. */
int hlbl_kernel_sum(hlbl_ctx* ctx, const double* d_fwd_src, const double* d_fwd_y,
                    const int gsx[4], const int yv[4], double xunit, int precision,
                    double out[2]);

/* As hlbl_kernel_sum, but asynchronous on the context's stream: the two
 * sums are written to d_out[2] (device) when the stream reaches them. */
int hlbl_kernel_sum_async(hlbl_ctx* ctx, const double* d_fwd_src, const double* d_fwd_y,
                          const int gsx[4], const int yv[4], double xunit, int precision,
                          double* d_out);

/* The kernel sums of n pairs that share the block y (the pairs one newly
 * solved source closes): pair i is (x = gsx[i], y = gsx[i] + yv[i]) with
 * the partner block srcs[i] (host array of device pointers); both flavours
 * to d_out[2*i..2*i+1] (device). Pairs run in batched launches of up to 16
 * (hlbl_ctx_set_batch_group): the pairs of a launch walk y's tiles in step,
 * so L2 can serve y to the partners after the first; each pair's CTAs still
 * read y themselves, and as the kernels are bound by arithmetic rather than
 * HBM, the autotuner usually keeps one pair per launch.
 * Asynchronous on the context's stream; capturable into a CUDA graph.
 * The per-source batching of the driver's pair loop (src/driver.cpp:104-134),
 * which calls Contractor::kernel_sum once per pair. */
int hlbl_kernel_sums_batched(hlbl_ctx* ctx, const double* d_fwd_y, int n,
                             const double* const* d_fwd_src, const int* gsx, const int* yv,
                             double xunit, int precision, double* d_out);
/* Pairs per batched launch (1..16; 0 = 16). */
int hlbl_ctx_set_batch_group(hlbl_ctx* ctx, int group);
/* Allocate the per-pair work buffers for batches of max_pairs (<= 16) now,
 * so that later calls allocate nothing (graph capture needs this). */
int hlbl_ctx_reserve(hlbl_ctx* ctx, int max_pairs);

/* Host-cache staging (PropagatorCache::device_ptr in host mode,
 * src/propagator_cache.cpp:52-68, which copies synchronously): copy `bytes`
 * from pinned host memory to d_dst on the context's side stream; the next
 * contraction call on the context waits for it, so a block can be staged
 * while the previous source's pairs are computed. With after_compute set the
 * copy first waits for all contraction work already enqueued on the
 * context (d_dst may still be read by it, as a reused staging slot is);
 * with it clear the caller guarantees that nothing enqueued reads d_dst. */
int hlbl_stage_async(hlbl_ctx* ctx, void* d_dst, const void* h_src, size_t bytes,
                     int after_compute);

/* Autotuner: times one batch (FP32 products) under each FP32 variant of
 * pass 1 (best_p1: 0 = tiles of 8 sites, 1 = 4) and pass 2 (best_p2:
 * 0 = CUDA cores, tiles of 4 sites; 1 = CUDA cores, 2 sites; 2 = tensor
 * cores) and each batch group (1, 2, 4, 8, 16 pairs per launch) and keeps
 * the fastest in the context. Writes the sums of the last trial to d_out.
 * Blocking. No counterpart in the reference. */
int hlbl_autotune(hlbl_ctx* ctx, const double* d_fwd_y, int n, const double* const* d_fwd_src,
                  const int* gsx, const int* yv, double xunit, double* d_out, int* best_p1,
                  int* best_p2, int* best_group, double* best_ms);

/* The FP32 tile copy of a block that pass 1 of the FP32 path writes and the
 * tensor-core pass 2 and hlbl_kernel_sums_batched_f32 read:
 * d_out[f][ia][tile][half][6][16][4] floats, tiles of 32 sites ((V + 31) / 32
 * of them, the last padded and its pad left untouched) in two halves of 16, a
 * site's 24 sink components as six groups of 4; each value rounded to
 * nearest even from FP64, 2 * 12 * tiles * 768 floats, then a trailer of 32
 * floats whose first two hold the largest magnitude of flavour 0 and 1
 * (hlbl_f32_block_length floats in all). Asynchronous on the context's
 * stream. No counterpart in the reference. */
int hlbl_f32_tile_copy(hlbl_ctx* ctx, const double* d_block, float* d_out);

/* Floats in one FP32 tile copy of a block of the context's lattice. */
size_t hlbl_f32_block_length(const hlbl_ctx* ctx);

/* hlbl_kernel_sums_batched on FP32 tile copies of the blocks (hlbl_f32_tile_copy,
 * made once per block when it enters the propagator cache): FP32 products
 * (pass 1 on the copies, pass 2 on the tensor cores), FP64 sums, the FP32
 * path's exact QED weight or the surrogate. Pair i = (gsx[i], gsx[i] + yv[i])
 * with partner copy x32s[i]; sums to d_out[2*i], [2*i+1]. Asynchronous on the
 * context's stream. No counterpart in the reference (the block format of the
 * reference's cache is FP64 only). */
int hlbl_kernel_sums_batched_f32(hlbl_ctx* ctx, const float* d_y32, int n, const float* const* d_x32s,
                                 const int* gsx, const int* yv, double xunit, double* d_out);

/* Autotuner of the FP32-copy path: pass-1 variant (0: both flavours per CTA,
 * one stage, two CTAs per SM; 1: both flavours, two stages, one CTA per SM;
 * 2: one flavour per CTA, two stages, three CTAs per SM; 3: as 2 with a
 * producer warp and per-stage empty/full barriers) and pairs per launch
 * (1, 2, 4, 8, 16),
 * timed on one batch; keeps the fastest. Blocking. No counterpart in the
 * reference. */
int hlbl_autotune_f32(hlbl_ctx* ctx, const float* d_y32, int n, const float* const* d_x32s,
                      const int* gsx, const int* yv, double xunit, double* d_out, int* best_variant,
                      int* best_group, double* best_ms);
/* Set what hlbl_autotune_f32 chooses: the pass-1 variant (0-3 as above)
 * and the pairs per launch (0: 16). */
int hlbl_ctx_set_p1f32_variant(hlbl_ctx* ctx, int variant, int group);

/* Exact QED weight of the FP32 path: the quadrature in FP32 where
 * min(|x|, |y|) >= r64 (units of 1/m_mu) and in FP64 inside (on = 1, the
 * default, r64 = 0.1), or FP64 everywhere (on = 0). The FP64 path always
 * evaluates it in FP64. No counterpart in the reference. */
int hlbl_ctx_set_qed_fp32(hlbl_ctx* ctx, int on, double r64);

/* FP32 two-flavour pass 2 on the tensor cores (on = 1, the default:
 * tcgen05 MMAs with split hi + lo products, FP32 tile copies of the blocks
 * written by pass 1 or by hlbl_f32_tile_copy; the operand type as
 * hlbl_ctx_set_tc_fp16 sets it, TF32 for FP64 blocks) or on the CUDA cores
 * (on = 0). No counterpart in the reference. */
int hlbl_ctx_set_tensor_cores(hlbl_ctx* ctx, int on);

/* Operands of the FP32-copy path's tensor-core pass 2 (hlbl_kernel_sums_batched_f32):
 * on = 1 (the default), FP16: the same hi + lo split as 3xTF32 (22
 * significant bits) in half the bytes and half the MMAs, with power-of-two
 * scales from the largest magnitudes the tile copies carry, so the copies
 * must come from hlbl_f32_tile_copy; on = 0, TF32. No counterpart in the
 * reference. */
int hlbl_ctx_set_tc_fp16(hlbl_ctx* ctx, int on);

/* One CUDA graph per window: every asynchronous call made on the context
 * between hlbl_graph_begin and hlbl_graph_end (typically one
 * hlbl_kernel_sums_batched per new source of a window) is recorded, not run;
 * hlbl_graph_launch replays it. Buffers are reserved for 16-pair batches at
 * begin. The recorded calls keep their pointers and arguments. */
typedef struct hlbl_graph hlbl_graph;
int hlbl_graph_begin(hlbl_ctx* ctx);
int hlbl_graph_end(hlbl_ctx* ctx, hlbl_graph** out);
int hlbl_graph_launch(hlbl_graph* graph, void* stream);
void hlbl_graph_destroy(hlbl_graph* graph);

/* Pass 1 of one flavour, ADDED into d_dzu[6][12][12][2] and
 * d_dzsu[4][12][12][2] (the caller zeroes them first). Same arguments and
 * meaning as the vendored launcher cu_dzu_dzsu (kernels/cuda_lattice.h:49-52,
 * kernels/cuda_lattice.cu:792-814); asynchronous. */
int hlbl_cu_dzu_dzsu(hlbl_ctx* ctx, double* d_dzu, double* d_dzsu, const double* fwd_src,
                     const double* fwd_y, int iflavor, const int proc_coords[4],
                     const int gsx[4], const int global_geom[4], const int local_geom[4]);

/* Pass 2 of one flavour, ADDED into *d_kernel_sum. g_dzu[6][4][12][24] and
 * g_dzsu[4][4][12][24] are pass 1's sums with gamma_mu gamma_5 inserted, as
 * contract.cpp:58-77 builds them. Same arguments and meaning as
 * cu_4pt_contraction (kernels/cuda_lattice.h:53-57, cuda_lattice.cu:816-839);
 * xunit is Pair::a (Pair::b is unused there too). Asynchronous. */
int hlbl_cu_4pt_contraction(hlbl_ctx* ctx, double* d_kernel_sum, const double* d_g_dzu,
                            const double* d_g_dzsu, const double* fwd_src,
                            const double* fwd_y, int iflavor, const int proc_coords[4],
                            const int gsx[4], double xunit, const int yv[4],
                            const int global_geom[4], const int local_geom[4]);

/* Pass 1 of one flavour, as hlbl_cu_dzu_dzsu, for callers that cannot
 * allocate device memory when they contract: for example a process whose
 * solver has already taken nearly all device memory into its own pool, or
 * one that measures free memory around the kernels. It needs no context and
 * allocates nothing. Its scratch (per-thread-block partial sums) is a fixed
 * array of HLBL_NOALLOC_MAX_BLOCKS x 2880 doubles (11.8 MB) in the library's
 * device image, held on every GPU that loads the library until exit; pass 1
 * walks the lattice's tiles with at most that many thread blocks, so every
 * lattice size fits. Runs on `stream` (a cudaStream_t; NULL = legacy
 * default) on the current device. The first call on a device looks up the
 * array's device address and the kernel's occupancy, so make that first call
 * before any stream capture. If a thread block gives up its bounded wait for
 * a staged tile, every element added into d_dzu and d_dzsu is NaN (the call
 * itself has returned HLBL_OK by then). All calls share the array and its
 * error word: calls that overlap on the GPU (other streams, other host
 * threads) race and give wrong sums; order them. No counterpart in the
 * reference. */
#define HLBL_NOALLOC_MAX_BLOCKS 512
int hlbl_cu_dzu_dzsu_noalloc(double* d_dzu, double* d_dzsu, const double* fwd_src,
                             const double* fwd_y, int iflavor, const int proc_coords[4],
                             const int gsx[4], const int global_geom[4],
                             const int local_geom[4], void* stream);

/* The gamma insertion of Contractor::compute_dzu_dzsu (contract.cpp:58-77)
 * on the device: g_dzu, g_dzsu from dzu, dzsu (one flavour). Asynchronous. */
int hlbl_insert_gammas(hlbl_ctx* ctx, const double* d_dzu, const double* d_dzsu,
                       double* d_g_dzu, double* d_g_dzsu);

/* ---- 2+2 pieces ----------------------------------------------------------
 * The 2+2 pieces of the source w = gsw for n_y targets (global sites in
 * [0, L)), from the device block of w (block_length doubles), this rank's
 * part (with more than one rank the caller sums over ranks, as
 * compute_2p2_gpu's MPI_Iallreduce does, kernels/hlbl_kernels/kernels.cu:824-860):
 *   P1   [4][4][4][Lmax]  P1[rho][sigma][nu][zeta] = sum of Pi(z)[sigma][nu]
 *                         over the sites with (z - w)_rho mod L_rho = zeta
 *                         (0 for zeta >= L_rho), Lmax = hlbl_2p2_lmax
 *   P234 P2_0, P2_1, P3, P4_0, P4_1 [rho][sigma][nu] per target, rho < sigma
 *                         (P4_1: rho != sigma), zero elsewhere
 * with Pi(z)[mu][nu] = Re sum_ia (g_nu g5 <d_ib, g5 g_mu u_ia>)[ia] of
 * u = fwd[iflavor], d = fwd[1 - iflavor] (kernel_pi, kernels.cu:241-294).
 * precision HLBL_FP64: FP64 throughout; HLBL_FP32: FP32 products and QED
 * weight (the FP64 weight where a kernel argument is shorter than
 * hlbl_ctx_set_2p2_r64's radius, by default nowhere), FP64 sums. */
/* The last dimension of P1: the largest global extent. */
int hlbl_2p2_lmax(const hlbl_ctx* ctx);
/* FP32 2+2 path: evaluate the QED weight in FP64 where min(|a|, |b|) of its
 * two arguments (units of 1/m_mu) is below r64; 0 (the default): nowhere. */
int hlbl_ctx_set_2p2_r64(hlbl_ctx* ctx, double r64);
/* Allocate the 2+2 work buffers now, so that later calls allocate nothing
 * (graph capture needs this). */
int hlbl_2p2_reserve(hlbl_ctx* ctx);
/* Contractor::pieces_2p2 (src/contract.cpp:116-156; include/hlbl/contract.hpp:54-56):
 * flavour 0, P234 per target, p234[n_y][5][64]; host arrays; blocking. */
int hlbl_pieces_2p2(hlbl_ctx* ctx, const double* d_fwd, const int gsw[4], const int* targets,
                    int n_y, double xunit, int precision, double* p1, double* p234);
/* As hlbl_pieces_2p2, asynchronous on the context's stream, device outputs
 * d_p1 [4][4][4][Lmax] and d_p234 [n_y][5][64]; capturable into a CUDA
 * graph after hlbl_2p2_reserve. */
int hlbl_pieces_2p2_async(hlbl_ctx* ctx, const double* d_fwd, const int gsw[4], const int* targets,
                          int n_y, double xunit, int precision, double* d_p1, double* d_p234);
/* As hlbl_pieces_2p2_async with precision HLBL_FP32, from the block's FP32
 * tile copy (hlbl_f32_tile_copy; hlbl_f32_block_length floats, 16-byte
 * aligned) instead of the FP64 block: where the copy exists already (the
 * FP32 kernel-sum path makes one per source), Pi reads half the bytes and
 * converts nothing. */
int hlbl_pieces_2p2_f32(hlbl_ctx* ctx, const float* d_x32, const int gsw[4], const int* targets,
                        int n_y, double xunit, double* d_p1, double* d_p234);
/* compute_2p2_gpu (kernels/hlbl_kernels/kernels.cu:753-870, declared at
 * kernels.cuh:10-13) without its MPI reduction: host P1 [4][4][4][Lmax] and
 * P234 in its own layout [5][n_y][64] (geometry first), flavour iflavor,
 * targets gycoords[n_y][4]; blocking. */
int hlbl_compute_2p2(hlbl_ctx* ctx, const double* d_fwd_y, double* P1, double* P234, int iflavor,
                     const int gsw[4], const int* gycoords, int n_y, double xunit, int precision);

/* Warm-launches every kernel variant on a 2^4 lattice and returns the device
 * bytes that took (Contractor::reserve_kernel_memory, contract.cpp:158-197). */
int hlbl_reserve_kernel_memory(hlbl_ctx* ctx, size_t* bytes);

/* Propagator fixtures on the device (RandomProvider, src/provider.cpp:25-69):
 * the reference's uniform [-1,1) field (bit-identical to the host one) and
 * the i.i.d. complex Gaussian field of the benchmark configurations. `seed`
 * is the per-source seed (hlbl_source_seed). Asynchronous. */
int hlbl_fill_random_block(hlbl_ctx* ctx, double* d_out, uint64_t seed);
int hlbl_fill_gaussian_block(hlbl_ctx* ctx, double* d_out, uint64_t seed);
uint64_t hlbl_source_seed(uint64_t run_seed, const int gsx[4]);

/* ---- the learned QED weight ---------------------------------------------
 * An MLP (3 -> 128 -> 128 -> 128 -> 6, SiLU, BF16 weights and activations,
 * FP32 accumulation on the tensor cores) that corrects a coarse 8-node FP32
 * quadrature of the six weight functions: w_j = base_j exp(sigma_j net_j
 * env(max(|x|,|y|))), env the radial envelope of the base's log-residual.
 * Trained on the GPU by the library's own forward/backward kernels on
 * samples labelled by the exact FP64 weight; the exact tensor assembly is
 * kept; outside the validated region (min(|x|,|y|) < r0 or max(|x|,|y|) >
 * r1, units of 1/m_mu) pass 2 uses the exact FP64 weight. No counterpart in the
 * reference (the task's learned-weight extension). */
#define HLBL_SURROGATE_NPARAM 34310
typedef struct hlbl_surrogate hlbl_surrogate;
typedef struct {
  long long n_samples; /* training samples, X, Y uniform in [0, radius], c in [-1, 1] */
  int batch;           /* rows per optimiser step */
  int steps;           /* Adam steps (cosine learning-rate decay to 1% of lr) */
  float lr;            /* initial learning rate */
  uint64_t seed;       /* sample seed */
  float radius;        /* training radius, units of 1/m_mu (6.43 = 12 fm) */
  long long n_valid;   /* validation samples (0: no validation, r0 = 0) */
  double bound;        /* per-weight relative error bound of the accepted region */
} hlbl_train_config;
typedef struct {
  float final_loss;          /* last step's loss (normalised targets) */
  double max_rel_err_net;    /* validation, outside r0: base x net vs exact */
  double rms_rel_err_net;
  double max_rel_err_base;   /* the same for the coarse base alone */
  double rms_rel_err_base;
  double r0;                 /* exact inside: min(|x|, |y|) < r0 */
  double train_seconds;      /* sample generation + training + validation */
  double r1;                 /* exact outside: max(|x|, |y|) > r1 */
} hlbl_train_report;
int hlbl_surrogate_create(hlbl_surrogate** out, int device, double lambda, uint64_t seed);
void hlbl_surrogate_destroy(hlbl_surrogate* s);
int hlbl_surrogate_train(hlbl_surrogate* s, const hlbl_train_config* cfg, hlbl_train_report* rep);
/* Host copies of the FP32 parameters [HLBL_SURROGATE_NPARAM] and the six
 * output scales: read (set = 0) or write (set = 1). */
int hlbl_surrogate_params(hlbl_surrogate* s, float* params, float* sigma, int set);
/* One forward + backward pass on host rows feat[n][3] (normalised inputs)
 * and targets[n][6] (normalised): gradients of the mean squared error in
 * the parameter layout, and the loss. The training step, exposed for the
 * gradient check. */
int hlbl_surrogate_gradients(hlbl_surrogate* s, const float* feat, const float* target, int n,
                             float* grad, float* loss);
/* The inference kernel's raw network outputs for host rows feat[n][3]. */
int hlbl_surrogate_eval(hlbl_surrogate* s, const float* feat, int n, float* out);
/* ---- the QED kernel ------------------------------------------------------
 * Which QED kernel pass 2 and the 2+2 pieces weight with. KQED's
 * QED_Mkernel_L2 (kernels/cuda_lattice.cu:266-275, kernels.cu:238) is not
 * available, so the library carries two test kernels with its signature
 * (include/hlbl_gb300_qed.h):
 *   HLBL_QEDK_STANDIN          the stand-in through its closed-form fast
 *                              paths (the default)
 *   HLBL_QEDK_STANDIN_GENERIC  the same tensor through the generic paths
 *   HLBL_QEDK_DENSE            the dense test weight (no index structure,
 *                              table seeded by `seed`), generic paths, entry
 *                              by entry
 *   HLBL_QEDK_DENSE_KERV       the same tensor evaluated whole per call, as
 *                              a QED_Mkernel_L2-shaped function is
 *   HLBL_QEDK_KQED             a linked KQED's QED_Mkernel_L2 (device code of
 *                              libKQED_cuda.a; a library built with
 *                              HLBL_KQED_DIR set; HLBL_EINVAL otherwise),
 *                              KQED's initialise() on first selection
 * The generic paths use no structure of the tensor: a coefficient stage
 * folds the three evaluations per site into 640 coefficients in HBM (FP32
 * or FP64 by the path), which the contraction kernels dot with their F rows,
 * and the 2+2 kernels contract all 384 entries per evaluation. The learned
 * weight (hlbl_ctx_set_qed) replaces the stand-in's closed form only.
 * Blocking. No counterpart in the reference (it links one kernel). */
enum { HLBL_QEDK_STANDIN = 0, HLBL_QEDK_STANDIN_GENERIC = 1, HLBL_QEDK_DENSE = 2,
       HLBL_QEDK_DENSE_KERV = 3, HLBL_QEDK_KQED = 4 };
int hlbl_ctx_set_qed_kernel(hlbl_ctx* ctx, int kind, uint64_t seed);

/* Pass 2's QED weight: HLBL_QED_EXACT, or HLBL_QED_SURROGATE with `s` and
 * fallback radius r0 (r0 < 0: the radius the training validation chose). */
int hlbl_ctx_set_qed(hlbl_ctx* ctx, int mode, hlbl_surrogate* s, double r0);
/* (site, evaluation) rows that pass 2 evaluated exactly, outside the
 * surrogate's validated region (within r0 of the origin or beyond the
 * largest radius its validation accepted), summed since the mode was set.
 * Those rows get the exact weight as the FP32 path has it (hlbl_ctx_set_qed_fp32):
 * the FP32 quadrature away from the origin, FP64 within r64 of it. */
int hlbl_ctx_qed_fallbacks(hlbl_ctx* ctx, unsigned long long* n);

/* Measurement hooks. With profiling on, the context times every pass-1 and
 * pass-2 contraction kernel with CUDA events on its launching stream;
 * hlbl_ctx_kernel_times returns the summed milliseconds and launch counts
 * ([0] pass 1, [1] pass 2) since profiling was switched on. */
int hlbl_ctx_set_profiling(hlbl_ctx* ctx, int on);
int hlbl_ctx_kernel_times(hlbl_ctx* ctx, double ms[2], long long n[2]);
/* FMA throughput of the CUDA cores (TFLOP/s, precision HLBL_FP64 or
 * HLBL_FP32), from a kernel of independent FMA chains. */
int hlbl_measure_fma_peak(int device, int precision, double* tflops);

/* Device doubles in one propagator block of this rank. */
size_t hlbl_block_length(const hlbl_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* HLBL_GB300_H */
