// peak.cu -- FMA throughput of this GPU's CUDA cores, FP64 and FP32: the
// compute roof the contraction kernels are reported against (the measured
// peaks supplied with the machine cover HBM and bf16 tensor throughput only).
#include <cuda_runtime.h>

#include "hlbl_gb300.h"
#include "hlbl_internal.h"

namespace {

// Each thread runs 8 independent FMA chains of `iters` steps; the chains
// keep the pipe full without depending on memory.
template <typename T>
__global__ void fma_peak_kernel(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = (T)(threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = x[i] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if (s == (T)-12345.678) out[0] = s;  // keeps the chains live
}

template <typename T>
int run_peak(int device, double* tflops) {
  int nsm = 0;
  cudaError_t e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return hg::cuda_fail(e, "SM count");
  T* out = nullptr;
  e = cudaMalloc(&out, sizeof(T));
  if (e != cudaSuccess) return hg::cuda_fail(e, "peak alloc");
  int const threads = 256, blocks = nsm * 8;
  int const iters = sizeof(T) == 8 ? 4096 : 65536;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fma_peak_kernel<T><<<blocks, threads>>>(out, iters / 16, (T)0.999, (T)0.001);  // warm-up
  cudaEventRecord(a);
  fma_peak_kernel<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(b);
  e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess) return hg::cuda_fail(e, "peak run");
  double const flop = 2.0 * 8.0 * iters * (double)threads * blocks;
  *tflops = flop / (ms * 1e-3) / 1e12;
  return HLBL_OK;
}

}  // namespace

extern "C" int hlbl_measure_fma_peak(int device, int precision, double* tflops) {
  if (!tflops) return hg::fail(HLBL_EINVAL, "hlbl_measure_fma_peak: null output");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return hg::cuda_fail(e, "cudaSetDevice");
  return precision == HLBL_FP64 ? run_peak<double>(device, tflops) : run_peak<float>(device, tflops);
}
