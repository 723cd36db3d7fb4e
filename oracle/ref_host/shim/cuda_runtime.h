/* Host-emulation shim of the CUDA runtime for building the reference's own
 * kernel and host sources as ordinary C++ (oracle/ref_host). Device memory is
 * host memory. Kernels whose launch the build strips (cuda_lattice.cu) run as
 * plain functions with one "thread" (the defaults below: blockDim = gridDim =
 * 1), so their grid-stride loops visit every site in order. Kernels launched
 * through hlbl_emu_launch (kernels.cu) run block after block, each block as
 * blockDim real threads with __syncthreads as a barrier, shared memory as
 * function statics (one block at a time) and warp shuffles exchanged through
 * per-warp barriers. Test infrastructure only. */
#pragma once
#include <barrier>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline
#define __restrict__
#define __shared__ static

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct hlbl_emu_uint3 { unsigned x, y, z; };
inline thread_local hlbl_emu_uint3 threadIdx{0, 0, 0};
inline thread_local hlbl_emu_uint3 blockIdx{0, 0, 0};
inline thread_local dim3 blockDim(1, 1, 1);
inline thread_local dim3 gridDim(1, 1, 1);

// the block the calling thread belongs to (null outside hlbl_emu_launch)
struct hlbl_emu_block {
  std::unique_ptr<std::barrier<>> bar;
  std::vector<std::unique_ptr<std::barrier<>>> warp;
  std::vector<double> lane_val;
  unsigned nthreads = 1;
};
inline thread_local hlbl_emu_block* hlbl_emu_cur = nullptr;
inline thread_local unsigned hlbl_emu_tid = 0;  // x + y Dx + z Dx Dy, as CUDA numbers lanes

inline void __syncthreads() {
  if (hlbl_emu_cur) hlbl_emu_cur->bar->arrive_and_wait();
}
inline unsigned __activemask() { return 0xffffffffu; }
// every lane of the warp calls it; a source lane past the warp returns the
// caller's own value, as on the device
inline double __shfl_down_sync(unsigned, double v, unsigned delta, int = 32) {
  hlbl_emu_block* b = hlbl_emu_cur;
  if (!b) return v;
  unsigned const w = hlbl_emu_tid / 32, lane = hlbl_emu_tid % 32;
  unsigned const wsize = (b->nthreads - 32 * w) < 32 ? (b->nthreads - 32 * w) : 32;
  b->lane_val[hlbl_emu_tid] = v;
  b->warp[w]->arrive_and_wait();
  double const r = lane + delta < wsize ? b->lane_val[hlbl_emu_tid + delta] : v;
  b->warp[w]->arrive_and_wait();
  return r;
}

// kernel<<<grid, block>>>(args) becomes hlbl_emu_launch(grid, block, [&]{ kernel(args); }):
// blockDim threads run the blocks one after another, with a barrier between
// blocks (the function statics that stand for shared memory are reused)
template <class F>
inline void hlbl_emu_launch(dim3 grid, dim3 block, F&& body) {
  unsigned const nt = block.x * block.y * block.z;
  hlbl_emu_block blk;
  blk.nthreads = nt;
  blk.bar = std::make_unique<std::barrier<>>((std::ptrdiff_t)nt);
  for (unsigned w = 0; w * 32 < nt; ++w)
    blk.warp.push_back(std::make_unique<std::barrier<>>((std::ptrdiff_t)(nt - 32 * w < 32 ? nt - 32 * w : 32)));
  blk.lane_val.assign(nt, 0.0);
  std::vector<std::thread> th;
  th.reserve(nt);
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      threadIdx = hlbl_emu_uint3{t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
      blockDim = block;
      gridDim = grid;
      hlbl_emu_cur = &blk;
      hlbl_emu_tid = t;
      for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
          for (unsigned bx = 0; bx < grid.x; ++bx) {
            blockIdx = hlbl_emu_uint3{bx, by, bz};
            body();
            blk.bar->arrive_and_wait();
          }
    });
  for (auto& x : th) x.join();
}

typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
  cudaMemcpyDeviceToDevice, cudaMemcpyDefault
};
inline const char* cudaGetErrorString(int e) { return e ? "emulated error" : "no error"; }
inline double atomicAdd_system(double* a, double v) {
  static std::mutex m;
  std::lock_guard<std::mutex> g(m);
  double o = *a;
  *a = o + v;
  return o;
}
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
typedef struct hlbl_emu_stream* cudaStream_t;
inline cudaError_t cudaStreamCreate(cudaStream_t* s) { *s = nullptr; return cudaSuccess; }
inline cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, std::size_t n, cudaMemcpyKind, cudaStream_t = nullptr) {
  std::memcpy(d, s, n);
  return cudaSuccess;
}
