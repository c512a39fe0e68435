// Instances of the Gray-code enumeration kernel for int64 coefficients and
// 9 inner bits, with their host-side launchers (one instruction variant:
// the three-input add and min of MODE 0).
#include "exhaustive_kernels.cuh"

namespace os {
namespace exh {

template <>
void launch_gray_width<long long, 9>(int, bool collect, int grid, cudaStream_t s, const GrayParams<long long> &P) {
  if (collect)
    gray_kernel<long long, 9, true, 0><<<grid, THREADS, 0, s>>>(P);
  else
    gray_kernel<long long, 9, false, 0><<<grid, THREADS, 0, s>>>(P);
  OS_CUDA(cudaGetLastError());
}

template <>
int gray_occupancy_width<long long, 9>(int) {
  int occ = 0;
  OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<long long, 9, false, 0>, THREADS, 0));
  return occ < 1 ? 1 : occ;
}

}  // namespace exh
}  // namespace os
