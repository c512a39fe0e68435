// philox.cuh -- counter-based Philox4x32-10 for the annealing kernels.
//
// Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw ("Parallel
// random numbers: as easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64
// multiplies with the published multipliers and Weyl key increments. The
// reference draws from oneMKL's philox4x32x10 engine
// (include/simulated_annealing/annealing.hpp:87); this generator is keyed by
// the caller's seed and countered by (site group, step, trajectory,
// instance), so every draw is a pure function of where it is used and no
// trajectory's stream overlaps another's.
#ifndef ONESOLVER_PHILOX_CUH_
#define ONESOLVER_PHILOX_CUH_

#include <cstdint>

namespace os {

struct Philox4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1,
                                                          uint32_t c2, uint32_t c3,
                                                          uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
    uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
#else
    uint64_t p0 = (uint64_t)M0 * c0, p1 = (uint64_t)M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  return Philox4{c0, c1, c2, c3};
}

// Uniform in (0, 1): (r + 0.5) * 2^-32 in FP32, never 0 or 1 after rounding
// of the 24-bit-precise result is clamped below 1.
__device__ __forceinline__ float u01_open(uint32_t r) {
  float u = ((float)(r >> 8) + 0.5f) * 0x1.0p-24f;
  return u;
}

// Streams of the annealing kernels (counter word c3's top bits).
enum : uint32_t {
  kStreamInit = 0x1u << 28,    // initial spins
  kStreamSweep = 0x2u << 28,   // acceptance uniforms (sequential sites)
  kStreamSite = 0x3u << 28,    // site index + uniform (random sites)
  kStreamExchange = 0x4u << 28,  // replica-exchange uniforms (tempering)
  kStreamResample = 0x5u << 28,  // resampling offsets (population annealing)
};

// Uniform in (0, 1) in FP64 from one 32-bit word: (r + 0.5) * 2^-32, exact.
__host__ __device__ __forceinline__ double u01_open64(uint32_t r) {
  return ((double)r + 0.5) * 0x1.0p-32;
}

}  // namespace os

#endif  // ONESOLVER_PHILOX_CUH_
