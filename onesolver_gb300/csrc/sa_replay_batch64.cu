// sa_replay_batch64.cu -- the REPLAY batched sweep kernel's 64-slot class,
// the slowest to compile, in a translation unit of its own (see
// sa_batch_tile.cuh).
#include "sa_batch_tile.cuh"

namespace os {
namespace sa {

template void batch_tile_op<64, true>(BatchTileOp, const BatchArgs *, int, int, size_t, cudaStream_t, int *);

}  // namespace sa
}  // namespace os
