// Launcher of the tile kernels of the OR-AND ring (one translation unit per ring and kernel
// family, compiled in parallel).
#include "tsg_tree_launch.cuh"

namespace tsg {
namespace dev {

tsg_status launch_tile_or_and(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  launch_tile_ring<TSG_RING_OR_AND>(la, ra, st);
  return TSG_OK;
}

}  // namespace dev
}  // namespace tsg
