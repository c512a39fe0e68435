// rescore.cuh -- the reference's FP64 energy function on the device.
//
// sa::energy (include/simulated_annealing/annealing.hpp:31-40) and the
// exhaustive inner loop (include/exhaustive/exhaustive.hpp:112-129) both sum
// F[i][j] over i <= j in row-major order, adding F[i][j] * x_i * x_j. The
// products by 0/1 are exact and adding a zero leaves any FP64 partial sum
// unchanged, so summing only the set pairs in the same order reproduces the
// reference's value bit for bit. The loop is serial on purpose.
#ifndef ONESOLVER_RESCORE_CUH_
#define ONESOLVER_RESCORE_CUH_

#include <cstdint>

namespace os {

__device__ __forceinline__ double rescore_energy(const double *__restrict__ f, int n,
                                                 const uint8_t *__restrict__ x) {
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    if (!x[i]) continue;
    const double *row = f + (size_t)i * n;
    e += row[i];
    for (int j = i + 1; j < n; ++j)
      if (x[j]) e += row[j];
  }
  return e;
}

// Same sum for a state held as bits (bit i = variable i), n <= 64.
__device__ __forceinline__ double rescore_energy_bits(const double *__restrict__ f, int n,
                                                      uint64_t s) {
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    if (!((s >> i) & 1ull)) continue;
    const double *row = f + (size_t)i * n;
    e += row[i];
    uint64_t rest = (i + 1 < 64) ? (s >> (i + 1)) : 0ull;
    int j = i + 1;
    while (rest) {
      int z = __ffsll((long long)rest) - 1;
      j += z;
      e += row[j];
      rest >>= z;
      rest >>= 1;
      j += 1;
    }
  }
  return e;
}

// Warp-parallel FP64 energy of one state, called by all 32 lanes of a warp
// (the result is returned in every lane). The spins are packed into `xw`
// (ceil(n / 32) words of shared memory private to the warp); lane l then sums
// F[i][j] over the set pairs i <= j with j = l mod 32, rows in order, and the
// lanes' partial sums are reduced with shuffles. Same terms as the
// reference's sum in a different order: coalesced row reads instead of one
// serial chain, at an FP64 rounding difference of a few ulps of the sum of
// the absolute terms.
__device__ __forceinline__ double rescore_energy_warp(const double *__restrict__ f, int n,
                                                      const uint8_t *__restrict__ x, unsigned *xw) {
  const int lane = threadIdx.x & 31;
  const int nw = (n + 31) >> 5;
  for (int k = 0; k < nw; ++k) {
    const int j = k * 32 + lane;
    const unsigned b = __ballot_sync(0xffffffffu, j < n && x[j]);
    if (lane == 0) xw[k] = b;
  }
  __syncwarp();
  double acc0 = 0.0, acc1 = 0.0;
  for (int ki = 0; ki < nw; ++ki) {
    unsigned bits = xw[ki];
    while (bits) {
      const int i = ki * 32 + __ffs(bits) - 1;
      bits &= bits - 1;
      const double *row = f + (size_t)i * n + lane;
      int kj = ki;
      for (; kj + 1 < nw; kj += 2) {
        const unsigned w0 = xw[kj], w1 = xw[kj + 1];
        const int j0 = kj * 32 + lane;
        if (j0 >= i && ((w0 >> lane) & 1u)) acc0 += row[kj * 32];
        if (((w1 >> lane) & 1u)) acc1 += row[(kj + 1) * 32];
      }
      if (kj < nw) {
        const int j0 = kj * 32 + lane;
        if (j0 >= i && ((xw[kj] >> lane) & 1u)) acc0 += row[kj * 32];
      }
    }
  }
  double acc = acc0 + acc1;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  return acc;
}

void launch_rescore(const double *d_f, int n, const uint8_t *d_states, int m,
                    double *d_out, cudaStream_t stream);

// FP64 energies of m states with rescore_energy_warp (one warp per state).
void launch_rescore_warp(const double *d_f, int n, const uint8_t *d_states, int m,
                         double *d_out, cudaStream_t stream);

}  // namespace os

#endif  // ONESOLVER_RESCORE_CUH_
