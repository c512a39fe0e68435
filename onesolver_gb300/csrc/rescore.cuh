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

// Block-parallel FP64 energy of one state, called by all threads of a CTA of
// RESCORE_WARPS warps (the result is returned in every thread). The spins are
// packed into `xw` (ceil(n / 32) words of shared memory); warp w takes the
// set rows i = w, w + RESCORE_WARPS, ... (in set-row order) and its lane l the
// columns j >= i with j = l mod 32, four row words in flight at a time; the
// partial sums meet in `red` (RESCORE_WARPS doubles of shared memory). Same
// terms as the reference's sum in a different order: coalesced row reads
// instead of one serial chain, at an FP64 rounding difference of a few ulps
// of the sum of the absolute terms.
constexpr int RESCORE_WARPS = 8;
__device__ __forceinline__ double rescore_energy_block(const double *__restrict__ f, int n,
                                                       const uint8_t *__restrict__ x, unsigned *xw, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (n + 31) >> 5;
  for (int k = warp; k < nw; k += RESCORE_WARPS) {
    const int j = k * 32 + lane;
    const unsigned b = __ballot_sync(0xffffffffu, j < n && x[j]);
    if (lane == 0) xw[k] = b;
  }
  __syncthreads();
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  int seen = 0;
  for (int ki = 0; ki < nw; ++ki) {
    unsigned bits = xw[ki];
    while (bits) {
      const int i = ki * 32 + __ffs(bits) - 1;
      bits &= bits - 1;
      if (seen++ % RESCORE_WARPS != warp) continue;
      const double *row = f + (size_t)i * n + lane;
      for (int kj = ki; kj < nw; kj += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = kj + u;
          if (k < nw && ((xw[k] >> lane) & 1u) && k * 32 + lane >= i) acc[u] += row[k * 32];
        }
      }
    }
  }
  double a = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
  if (lane == 0) red[warp] = a;
  __syncthreads();
  double e = 0.0;
#pragma unroll
  for (int w = 0; w < RESCORE_WARPS; ++w) e += red[w];
  return e;
}

void launch_rescore(const double *d_f, int n, const uint8_t *d_states, int m,
                    double *d_out, cudaStream_t stream);

// FP64 energies of m states with rescore_energy_block (one CTA per state).
void launch_rescore_warp(const double *d_f, int n, const uint8_t *d_states, int m,
                         double *d_out, cudaStream_t stream);

}  // namespace os

#endif  // ONESOLVER_RESCORE_CUH_
