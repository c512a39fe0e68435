// common.cuh -- shared plumbing of the C ABI: status handling, the
// thread-local error string, the execution context and small device helpers.
#ifndef ONESOLVER_COMMON_CUH_
#define ONESOLVER_COMMON_CUH_

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <tuple>

#include "onesolver.h"
#include "errors.hpp"

// A failed runtime call also leaves its error in the thread's last-error
// slot; clear it so that a later cudaGetLastError() check does not report a
// stale failure.
#define OS_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t err__ = (call);                                                \
    if (err__ != cudaSuccess) {                                                \
      (void)cudaGetLastError();                                                \
      ::os::throw_error(OS_CUDA_ERROR, "%s failed: %s (%s:%d)", #call,         \
                        cudaGetErrorString(err__), __FILE__, __LINE__);        \
    }                                                                          \
  } while (0)

namespace os {

// Device buffer owned by a plan or context (freed on destruction). alloc()
// takes memory from cudaMalloc; alloc_on() takes it stream-ordered from a
// memory pool (the context's, which keeps freed blocks cached), and the
// buffer is then freed in order on the same stream, so a later allocation
// of the same size on that stream reuses the block without a device-wide
// synchronisation.
template <class T> struct DevBuf {
  T *ptr = nullptr;
  size_t count = 0;
  cudaMemPool_t pool = nullptr;
  cudaStream_t stream = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) {
      if (pool)
        cudaFreeAsync(ptr, stream);
      else
        cudaFree(ptr);
    }
    ptr = nullptr;
    count = 0;
    pool = nullptr;
    stream = nullptr;
  }
  void alloc(size_t n) {
    if (n <= count && ptr && !pool) return;
    release();
    if (n == 0) n = 1;
    OS_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
    count = n;
  }
  void alloc_on(size_t n, cudaMemPool_t mp, cudaStream_t s) {
    if (n <= count && ptr && pool == mp && stream == s) return;
    release();
    if (n == 0) n = 1;
    OS_CUDA(cudaMallocFromPoolAsync(reinterpret_cast<void **>(&ptr), n * sizeof(T), mp, s));
    count = n;
    pool = mp;
    stream = s;
  }
  T *get() const { return ptr; }
};

}  // namespace os

// The execution context behind os_ctx.
struct os_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // Stream-ordered memory pool of the context's plans (DevBuf::alloc_on);
  // keeps up to 1 GiB of freed blocks for reuse.
  cudaMemPool_t pool = nullptr;
  // Tuned trajectories per CTA of the dense staged-tile sweep, keyed by
  // (padded row length, trajectories, acceptance rule): later plans of the
  // same shape reuse the choice instead of probing again.
  std::map<std::tuple<int, int, int>, int> dense_warps;
};

namespace os {

// Make the context's device current for the calling thread.
void activate(os_ctx *ctx);

__host__ __device__ inline uint64_t ceil_div_u64(uint64_t a, uint64_t b) {
  return (a + b - 1) / b;
}

}  // namespace os

#endif  // ONESOLVER_COMMON_CUH_
