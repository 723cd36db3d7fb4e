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
 * device image, held on every GPU that loads the library until exit; a call
 * whose pass 1 would run more thread blocks than that fails with
 * HLBL_EINVAL. Runs on `stream` (a cudaStream_t; NULL = legacy default) on
 * the current device. The first call on a device looks up the array's device
 * address and the kernel's occupancy, so make that first call before any
 * stream capture. All calls share the array: calls that overlap on the GPU
 * (other streams, other host threads) race and give wrong sums; order them.
 * No counterpart in the reference. */
#define HLBL_NOALLOC_MAX_BLOCKS 512
int hlbl_cu_dzu_dzsu_noalloc(double* d_dzu, double* d_dzsu, const double* fwd_src,
                             const double* fwd_y, int iflavor, const int proc_coords[4],
                             const int gsx[4], const int global_geom[4],
                             const int local_geom[4], void* stream);

/* The gamma insertion of Contractor::compute_dzu_dzsu (contract.cpp:58-77)
 * on the device: g_dzu, g_dzsu from dzu, dzsu (one flavour). Asynchronous. */
int hlbl_insert_gammas(hlbl_ctx* ctx, const double* d_dzu, const double* d_dzsu,
                       double* d_g_dzu, double* d_g_dzsu);

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
