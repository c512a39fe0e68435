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

void launch_rescore(const double *d_f, int n, const uint8_t *d_states, int m,
                    double *d_out, cudaStream_t stream);

}  // namespace os

#endif  // ONESOLVER_RESCORE_CUH_
