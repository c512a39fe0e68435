// probe.cu -- measured roofline denominators that the driver does not
// provide: the issue rate of the instructions each exhaustive variant spends
// per state (three-input add with a constant-bank operand and an integer
// min; multiply-add and fused add-min; packed 16-bit halves, a three-input
// add per two states and a three-input per-half min per four), the FP32 FMA
// rate, and the shared-memory read rate of the dense annealing row update
// (one 128-bit shared load feeding two paired FP32 FMAs per lane, the
// instruction pair of a field update).
#include <cstdint>
#include <utility>

#include "common.cuh"

namespace os {
namespace probe {

constexpr int STEPS = 256;
constexpr int CHAINS = 4;

struct ProbeParams {
  int k[STEPS];
  int iters;
  int *sink;
};

template <int I>
__device__ __forceinline__ void step(int (&E)[CHAINS], int (&m)[CHAINS], const int (&c)[CHAINS],
                                     const ProbeParams &P) {
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) {
    E[j] += P.k[I] + ((I & 1) ? c[j] : -c[j]);
    m[j] = min(m[j], E[j]);
  }
}

template <int... Is>
__device__ __forceinline__ void steps(int (&E)[CHAINS], int (&m)[CHAINS], const int (&c)[CHAINS],
                                      const ProbeParams &P, std::integer_sequence<int, Is...>) {
  (step<Is>(E, m, c, P), ...);
}

// Per iteration: STEPS * CHAINS (add, min) pairs = 2 * STEPS * CHAINS ops.
__global__ void __launch_bounds__(256) int32_probe_kernel(const __grid_constant__ ProbeParams P) {
  int E[CHAINS], m[CHAINS], c[CHAINS];
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) {
    E[j] = threadIdx.x * 7 + j;
    m[j] = 1 << 30;
    c[j] = (blockIdx.x + j) & 3;
  }
  for (int it = 0; it < P.iters; ++it) {
    steps(E, m, c, P, std::make_integer_sequence<int, STEPS>{});
#pragma unroll
    for (int j = 0; j < CHAINS; ++j) c[j] ^= m[j] & 1;
  }
  int r = 0;
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) r ^= m[j] ^ E[j];
  if (r == 0x7fffffff) P.sink[0] = r;
}

// The per-state instructions of exhaustive variant V (1: three-input add +
// min; 2: multiply-add + fused add-min; 3: packed 16-bit halves, one
// three-input add per two states and one three-input per-half min per four:
// the packed walk's whole inner loop), STEPS steps of CHAINS independent
// chains per thread; the step constants come from the parameter bank as in
// the enumeration kernel.
struct PairParams {
  int k[STEPS];
  int k2s[STEPS];
  int iters;
  int *sink;
};

template <int V, int I>
__device__ __forceinline__ void pair_step(int (&E)[CHAINS], int (&m)[CHAINS], const int (&c)[CHAINS],
                                          const PairParams &P, int pos, int neg) {
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) {
    if constexpr (V == 1) {
      E[j] += P.k[I] + ((I & 1) ? c[j] : -c[j]);
      m[j] = min(m[j], E[j]);
    } else if constexpr (V == 2) {
      E[j] = c[j] * ((I & 1) ? pos : neg) + E[j];
      m[j] = __viaddmin_s32(E[j], P.k[I], m[j]);
    } else {
      const int e1 = E[j];
      E[j] = E[j] + P.k2s[I] + ((I & 2) ? c[j] : -c[j]);
      if (I & 1) m[j] = (int)__vimin3_s16x2((unsigned)m[j], (unsigned)e1, (unsigned)E[j]);
    }
  }
}

template <int V, int... Is>
__device__ __forceinline__ void pair_steps(int (&E)[CHAINS], int (&m)[CHAINS], const int (&c)[CHAINS],
                                           const PairParams &P, int pos, int neg,
                                           std::integer_sequence<int, Is...>) {
  (pair_step<V, Is>(E, m, c, P, pos, neg), ...);
}

template <int V>
__global__ void __launch_bounds__(256) pair_probe_kernel(const __grid_constant__ PairParams P) {
  int E[CHAINS], m[CHAINS], c[CHAINS];
  const int pos = P.k[0] | 1, neg = -pos;  // runtime +-1 (k[0] = 1)
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) {
    E[j] = threadIdx.x * 7 + j;
    m[j] = 1 << 30;
    c[j] = (blockIdx.x + j) & 3;
  }
  for (int it = 0; it < P.iters; ++it) {
    pair_steps<V>(E, m, c, P, pos, neg, std::make_integer_sequence<int, STEPS>{});
#pragma unroll
    for (int j = 0; j < CHAINS; ++j) c[j] ^= m[j] & 1;
  }
  int r = 0;
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) r ^= m[j] ^ E[j];
  if (r == 0x7fffffff) P.sink[0] = r;
}

// Per iteration: 8 independent FMA chains x 64 steps.
__global__ void __launch_bounds__(256) fp32_probe_kernel(int iters, float a, float b, float *sink) {
  float v[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = threadIdx.x * 1e-3f + j;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int s = 0; s < 64; ++s)
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = fmaf(v[j], a, b);
  }
  float r = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) r += v[j];
  if (r == 1234.5f) sink[0] = r;
}

// Per iteration: four 128-bit shared loads (64 bytes) and eight paired
// FMAs per thread, from 16 rows of 512 floats (conflict-free: lane l reads
// floats 4l..4l+3 of each 128-float group, like the dense field update).
constexpr int ROW_PROBE_FLOATS = 16 * 512;
__global__ void __launch_bounds__(256) smem_row_probe_kernel(int iters, float sgn, float *sink) {
  __shared__ __align__(16) float buf[ROW_PROBE_FLOATS];
  for (int i = threadIdx.x; i < ROW_PROBE_FLOATS; i += blockDim.x) buf[i] = (float)(i & 1023) * 1e-4f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned long long s2 = ((unsigned long long)__float_as_uint(sgn) << 32) | __float_as_uint(sgn);
  unsigned long long acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = 0ull;
  for (int it = 0; it < iters; ++it) {
    const float *row = buf + ((it * 7 + warp) & 15) * 512 + 4 * lane;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(row + g * 128);
      asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc[2 * g]) : "l"(v.x), "l"(s2));
      asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc[2 * g + 1]) : "l"(v.y), "l"(s2));
    }
  }
  unsigned long long r = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) r ^= acc[j];
  if (r == 0x123456789abcdefull) sink[0] = 1.f;
}

template <class F> double time_ms(cudaStream_t s, F &&launch) {
  cudaEvent_t e0, e1;
  OS_CUDA(cudaEventCreate(&e0));
  OS_CUDA(cudaEventCreate(&e1));
  launch();  // warm-up
  OS_CUDA(cudaEventRecord(e0, s));
  launch();
  OS_CUDA(cudaEventRecord(e1, s));
  OS_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  OS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

}  // namespace probe
}  // namespace os

using namespace os;
using namespace os::probe;

extern "C" {

os_status os_probe_int32_peak(os_ctx *ctx, double *gops) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(gops != nullptr, "null output");
    DevBuf<int> sink;
    sink.alloc(1);
    ProbeParams P{};
    for (int i = 0; i < STEPS; ++i) P.k[i] = (i * 2654435761u) & 15;
    P.iters = 64;
    P.sink = sink.get();
    int occ = 0;
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, int32_probe_kernel, 256, 0));
    const int grid = ctx->sm_count * (occ > 0 ? occ : 1);
    const double ms = time_ms(ctx->stream, [&] {
      int32_probe_kernel<<<grid, 256, 0, ctx->stream>>>(P);
      OS_CUDA(cudaGetLastError());
    });
    const double ops = 2.0 * STEPS * CHAINS * (double)P.iters * grid * 256.0;
    *gops = ops / (ms * 1e-3) / 1e9;
  });
}

os_status os_probe_exhaustive_pair(os_ctx *ctx, int32_t variant, double *states_per_s) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(states_per_s != nullptr, "null output");
    OS_REQUIRE(variant >= 1 && variant <= 3, "variant must be 1, 2 or 3");
    DevBuf<int> sink;
    sink.alloc(1);
    PairParams P{};
    for (int i = 0; i < STEPS; ++i) {
      P.k[i] = i == 0 ? 1 : (int)((i * 2654435761u) & 15);
      P.k2s[i] = (int)((uint32_t)P.k[i] * 0x10001u);
    }
    P.iters = 64;
    P.sink = sink.get();
    auto kern = variant == 1 ? pair_probe_kernel<1> : variant == 2 ? pair_probe_kernel<2> : pair_probe_kernel<3>;
    int occ = 0;
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, 0));
    const int grid = ctx->sm_count * (occ > 0 ? occ : 1);
    const double ms = time_ms(ctx->stream, [&] {
      kern<<<grid, 256, 0, ctx->stream>>>(P);
      OS_CUDA(cudaGetLastError());
    });
    const double steps = (double)STEPS * CHAINS * (double)P.iters * grid * 256.0;
    *states_per_s = steps * (variant == 3 ? 2.0 : 1.0) / (ms * 1e-3);
  });
}

os_status os_probe_fp32_fma_peak(os_ctx *ctx, double *gflops) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(gflops != nullptr, "null output");
    DevBuf<float> sink;
    sink.alloc(1);
    int occ = 0;
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fp32_probe_kernel, 256, 0));
    const int grid = ctx->sm_count * (occ > 0 ? occ : 1);
    const int iters = 512;
    const double ms = time_ms(ctx->stream, [&] {
      fp32_probe_kernel<<<grid, 256, 0, ctx->stream>>>(iters, 0.999f, 0.001f, sink.get());
      OS_CUDA(cudaGetLastError());
    });
    const double flops = 2.0 * 64 * 8 * (double)iters * grid * 256.0;
    *gflops = flops / (ms * 1e-3) / 1e9;
  });
}

os_status os_probe_smem_row_peak(os_ctx *ctx, double *gbs) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(gbs != nullptr, "null output");
    DevBuf<float> sink;
    sink.alloc(1);
    int occ = 0;
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, smem_row_probe_kernel, 256, 0));
    const int grid = ctx->sm_count * (occ > 0 ? occ : 1);
    const int iters = 4096;
    const double ms = time_ms(ctx->stream, [&] {
      smem_row_probe_kernel<<<grid, 256, 0, ctx->stream>>>(iters, -1.f, sink.get());
      OS_CUDA(cudaGetLastError());
    });
    const double bytes = 64.0 * (double)iters * grid * 256.0;
    *gbs = bytes / (ms * 1e-3) / 1e9;
  });
}

}  // extern "C"
