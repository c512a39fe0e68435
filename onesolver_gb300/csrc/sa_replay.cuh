// sa_replay.cuh -- launchers of the replay (verification) instantiations of
// the dense and batched sweep kernels (sa_replay.cu and sa_replay_batch.cu,
// translation units of their own so that nvcc builds them beside the
// production kernels).
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

// The production batched kernel's launchers (sa_batch_tile.cu and
// sa_batch_tile64.cu, translation units of their own): one persistent
// launch, its shared-memory limit, its largest block and its CTAs per SM for
// W warps.
void batch_tile_launch(const BatchArgs &b, int slot_cls, int grid, size_t smem, cudaStream_t s);
void batch_tile_set_smem(int slot_cls, size_t smem);
void batch_tile_max_threads(int slot_cls, int *out);
void batch_tile_occupancy(int slot_cls, int W, size_t smem, int *occ);

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_REPLAY_CUH_
