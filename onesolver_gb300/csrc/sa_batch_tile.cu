// sa_batch_tile.cu -- the production batched sweep kernel's launchers
// (slot classes 4 to 32 instantiated here, 64 in sa_batch_tile64.cu), in a
// translation unit of their own so that the library's parallel build
// compiles them beside the batched plan's host code (sa_batch.cu).
#include "sa_batch_tile.cuh"
#include "sa_replay.cuh"

namespace os {
namespace sa {

void batch_tile_launch(const BatchArgs &b, int slot_cls, int grid, size_t smem, cudaStream_t s) {
  OS_BATCH_TILE_SWITCH(slot_cls, false, kBatchLaunch, &b, grid, 0, smem, s, nullptr);
}
void batch_tile_set_smem(int slot_cls, size_t smem) {
  OS_BATCH_TILE_SWITCH(slot_cls, false, kBatchSetSmem, nullptr, 0, 0, smem, nullptr, nullptr);
}
void batch_tile_max_threads(int slot_cls, int *out) {
  OS_BATCH_TILE_SWITCH(slot_cls, false, kBatchMaxThreads, nullptr, 0, 0, 0, nullptr, out);
}
void batch_tile_occupancy(int slot_cls, int W, size_t smem, int *occ) {
  OS_BATCH_TILE_SWITCH(slot_cls, false, kBatchOccupancy, nullptr, 0, W, smem, nullptr, occ);
}

}  // namespace sa
}  // namespace os
