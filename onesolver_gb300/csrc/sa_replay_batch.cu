// sa_replay_batch.cu -- the REPLAY instantiations of the batched sweep
// kernel (slot classes 4 to 32 here, 64 in sa_replay_batch64.cu), in
// translation units of their own so that the library's parallel build
// compiles them beside the dense ones (sa_replay.cu); see sa_replay.cu for
// the replay mode itself.
#include "sa_batch_tile.cuh"
#include "sa_replay.cuh"

namespace os {
namespace sa {

void batch_tile_replay(const BatchArgs &b, int slot_cls, int grid, size_t smem, cudaStream_t s) {
  OS_BATCH_TILE_SWITCH(slot_cls, true, kBatchLaunch, &b, grid, 0, smem, s, nullptr);
  OS_CUDA(cudaGetLastError());
}

void batch_replay_smem(int slot_cls, size_t smem) {
  OS_BATCH_TILE_SWITCH(slot_cls, true, kBatchSetSmem, nullptr, 0, 0, smem, nullptr, nullptr);
}

}  // namespace sa
}  // namespace os
