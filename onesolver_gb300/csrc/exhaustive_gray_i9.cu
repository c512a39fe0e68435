// Instances of the Gray-code enumeration kernel for int coefficients and
// 9 inner bits, with their host-side launchers.
#include "exhaustive_kernels.cuh"

namespace os {
namespace exh {

template <>
void launch_gray_width<int, 9>(int variant, bool collect, int grid, cudaStream_t s, const GrayParams<int> &P) {
  if (collect)
    gray_kernel<int, 9, true, 0><<<grid, THREADS, 0, s>>>(P);
  else if (variant == OS_EXH_VARIANT_PACKED)
    gray_kernel<int, 9, false, 2><<<grid, THREADS, 0, s>>>(P);
  else if (variant == OS_EXH_VARIANT_FUSED)
    gray_kernel<int, 9, false, 1><<<grid, THREADS, 0, s>>>(P);
  else
    gray_kernel<int, 9, false, 0><<<grid, THREADS, 0, s>>>(P);
  OS_CUDA(cudaGetLastError());
}

// Resident CTAs per SM of the instance that runs `variant`.
template <>
int gray_occupancy_width<int, 9>(int variant) {
  int occ = 0;
  if (variant == OS_EXH_VARIANT_PACKED)
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<int, 9, false, 2>, THREADS, 0));
  else if (variant == OS_EXH_VARIANT_FUSED)
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<int, 9, false, 1>, THREADS, 0));
  else
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<int, 9, false, 0>, THREADS, 0));
  return occ < 1 ? 1 : occ;
}

}  // namespace exh
}  // namespace os
