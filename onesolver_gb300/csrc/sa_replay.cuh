// sa_replay.cuh -- launchers of the replay (verification) instantiations of
// the dense and batched sweep kernels (sa_replay.cu, a translation unit of
// its own so that nvcc builds them beside the production kernels).
#ifndef ONESOLVER_SA_REPLAY_CUH_
#define ONESOLVER_SA_REPLAY_CUH_

#include <cstddef>

#include <cuda_runtime.h>

#include "sa_kernels.cuh"

namespace os {
namespace sa {

// dense_sweeps (sa_dense.cu) with the REPLAY kernels: the same choice of
// kernel (staged tiles for sequential sweeps up to TILE_MAX_LD, read-only
// rows above it, the random-site kernel) and the same launch shape.
void dense_sweeps_replay(const DenseArgs &a, int slot_cls, int warps, bool sequential, cudaStream_t s);

// One persistent launch of the REPLAY batched kernel (sa_batch.cu's launch
// shape); batch_replay_smem sets its shared-memory limit first.
void batch_tile_replay(const BatchArgs &b, int slot_cls, int grid, size_t smem, cudaStream_t s);
void batch_replay_smem(int slot_cls, size_t smem);

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_REPLAY_CUH_
