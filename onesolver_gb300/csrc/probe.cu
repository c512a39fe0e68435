// probe.cu -- measured roofline denominators beyond the HBM copy and bf16
// GEMM peaks: the rate of each exhaustive variant's own inner block walk (the
// enumeration kernel's instruction sequence without its bookkeeping), the
// INT32 add + min issue rate, the FP32 FMA rate, and the shared-memory read rate of the dense annealing row update
// (one 128-bit shared load feeding two paired FP32 FMAs per lane, the
// instruction pair of a field update).
#include <cstdint>
#include <utility>

#include <memory>

#include "common.cuh"
#include "exhaustive_kernels.cuh"

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

// The enumeration kernel's own inner block walk for exhaustive variant V
// (exh::inner_block, MODE 0 or 1, for variants 1 and 2;
// exh::inner_block_packed for the packed variant 3), one block of 2^G inner
// steps after another, each from couplings that the previous block's minimum
// changes -- as in the enumeration, where a walked-bit flip changes them
// between blocks, so that nothing can be hoisted out of the walk. Full
// occupancy at the kernel's own launch bounds, no per-item bookkeeping: the
// ceiling of this variant's instruction sequence. (A walk whose couplings
// never change lets the compiler move part of the adds to the FMA pipe; the
// enumeration's cannot, so such a walk is not this kernel's ceiling.)
constexpr int WALK_G = exh::G_DEFAULT;

template <int V>
__global__ void __launch_bounds__(exh::THREADS, 5) walk_probe_kernel(const __grid_constant__ exh::GrayParams<int> P,
                                                                     int iters, int *sink) {
  int c[WALK_G];
#pragma unroll
  for (int i = 0; i < WALK_G; ++i) c[i] = (int)(((threadIdx.x + blockIdx.x + i) & 3) * (V == 3 ? 65537u : 1u));
  int E0 = V == 3 ? (int)((16384u + (threadIdx.x & 255)) * 65537u) : (int)threadIdx.x;
  const int pos = P.one, neg = -P.one;
  int acc = 0;
  for (int it = 0; it < iters; ++it) {
    int m;
    if constexpr (V == 3) {
      m = exh::inner_block_packed<WALK_G>(E0, c, P);
    } else {
      int E = E0;
      m = E0;
      exh::inner_block<int, WALK_G, V - 1>(E, m, c, P, pos, neg);
    }
    acc ^= m;
    E0 += m & 1;
#pragma unroll
    for (int i = 0; i < WALK_G; ++i) c[i] += (m >> i) & (V == 3 ? 65537 : 1);
  }
  if (acc == 0x7fffffff) sink[0] = acc;
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
    auto P = std::make_unique<exh::GrayParams<int>>();
    for (int t = 0; t < exh::INNER_MAX; ++t) {
      P->kf[t] = t == 0 ? 0 : (int)((t * 2654435761u) >> 29) - 4;  // small step deltas in [-4, 3]
      P->ks[t] = t == 0 ? 0 : P->ks[t - 1] + P->kf[t];
      P->kp[t] = (int)((uint32_t)P->kf[t] * 65537u);
    }
    P->one = 1;
    const int iters = 64;
    auto kern = variant == 1 ? walk_probe_kernel<1> : variant == 2 ? walk_probe_kernel<2> : walk_probe_kernel<3>;
    int occ = 0;
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, exh::THREADS, 0));
    const int grid = ctx->sm_count * (occ > 0 ? occ : 1);
    const double ms = time_ms(ctx->stream, [&] {
      kern<<<grid, exh::THREADS, 0, ctx->stream>>>(*P, iters, sink.get());
      OS_CUDA(cudaGetLastError());
    });
    // Per block: 2^G inner states per walk, two walks in the packed variant.
    const double states = (double)(1 << WALK_G) * (variant == 3 ? 2.0 : 1.0) * iters * grid * exh::THREADS;
    *states_per_s = states / (ms * 1e-3);
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
