/* Host-emulation shim of the CUDA runtime for building the reference's own
 * kernel and host sources as ordinary C++ (oracle/ref_host). Kernels become
 * plain functions that run with one "thread" (blockDim = gridDim = 1), so
 * their grid-stride loops visit every site in order; device memory is host
 * memory. Test infrastructure only. */
#pragma once
#include <cstddef>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline
#define __restrict__

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct hlbl_emu_uint3 { unsigned x, y, z; };
inline const hlbl_emu_uint3 threadIdx{0, 0, 0};
inline const hlbl_emu_uint3 blockIdx{0, 0, 0};
inline const dim3 blockDim(1, 1, 1);
inline const dim3 gridDim(1, 1, 1);

typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
  cudaMemcpyDeviceToDevice, cudaMemcpyDefault
};
inline const char* cudaGetErrorString(int e) { return e ? "emulated error" : "no error"; }
inline double atomicAdd_system(double* a, double v) { double o = *a; *a = o + v; return o; }
inline cudaError_t cudaMalloc(void** p, std::size_t n) {
  *p = std::malloc(n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
template <class T> inline cudaError_t cudaMalloc(T** p, std::size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), n);
}
inline cudaError_t cudaMallocHost(void** p, std::size_t n) { return cudaMalloc(p, n); }
template <class T> inline cudaError_t cudaMallocHost(T** p, std::size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), n);
}
inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaFreeHost(void* p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, std::size_t n, cudaMemcpyKind) {
  std::memcpy(d, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemset(void* d, int v, std::size_t n) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaMemGetInfo(std::size_t* f, std::size_t* t) { *f = 0; *t = 0; return cudaSuccess; }
