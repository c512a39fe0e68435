// sa_batch_tile.cuh -- host-side operations on the batched sweep kernel of
// one slot class (launch, shared-memory limit, largest block, CTAs per SM).
// The kernel's compile time grows with its slot class, so the 64-slot class
// is instantiated explicitly in translation units of its own
// (sa_batch_tile64.cu, sa_replay_batch64.cu) and the dispatchers
// (sa_batch_tile.cu, sa_replay_batch.cu) only declare it: the library's
// parallel build compiles the classes side by side.
#ifndef ONESOLVER_SA_BATCH_TILE_CUH_
#define ONESOLVER_SA_BATCH_TILE_CUH_

#include "common.cuh"
#include "sa_kernels.cuh"

namespace os {
namespace sa {

enum BatchTileOp { kBatchLaunch, kBatchSetSmem, kBatchMaxThreads, kBatchOccupancy };

template <int SLOTS, bool REPLAY>
void batch_tile_op(BatchTileOp op, const BatchArgs *b, int grid, int W, size_t smem, cudaStream_t s, int *out) {
  switch (op) {
    case kBatchLaunch:
      sa_batch_tile_kernel<SLOTS, REPLAY><<<grid, b->W * 32, smem, s>>>(*b);
      break;
    case kBatchSetSmem:
      OS_CUDA(cudaFuncSetAttribute(sa_batch_tile_kernel<SLOTS, REPLAY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
      break;
    case kBatchMaxThreads: {
      cudaFuncAttributes attr;
      OS_CUDA(cudaFuncGetAttributes(&attr, sa_batch_tile_kernel<SLOTS, REPLAY>));
      *out = attr.maxThreadsPerBlock;
      break;
    }
    case kBatchOccupancy:
      OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, sa_batch_tile_kernel<SLOTS, REPLAY>, W * 32, smem));
      break;
  }
}

extern template void batch_tile_op<64, false>(BatchTileOp, const BatchArgs *, int, int, size_t, cudaStream_t,
                                              int *);
extern template void batch_tile_op<64, true>(BatchTileOp, const BatchArgs *, int, int, size_t, cudaStream_t,
                                             int *);

// The slot-class switch of both dispatchers.
#define OS_BATCH_TILE_SWITCH(cls, REPLAY, ...)                             \
  switch (cls) {                                                           \
    case 4: batch_tile_op<4, REPLAY>(__VA_ARGS__); break;                  \
    case 8: batch_tile_op<8, REPLAY>(__VA_ARGS__); break;                  \
    case 16: batch_tile_op<16, REPLAY>(__VA_ARGS__); break;                \
    case 32: batch_tile_op<32, REPLAY>(__VA_ARGS__); break;                \
    case 64: batch_tile_op<64, REPLAY>(__VA_ARGS__); break;                \
    default: throw_error(OS_INVALID_ARG, "unsupported slot count %d", cls); \
  }

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_BATCH_TILE_CUH_
