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

// Device buffer owned by a plan or context (freed on destruction).
template <class T> struct DevBuf {
  T *ptr = nullptr;
  size_t count = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
  void alloc(size_t n) {
    if (n <= count && ptr) return;
    release();
    if (n == 0) n = 1;
    OS_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
    count = n;
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
