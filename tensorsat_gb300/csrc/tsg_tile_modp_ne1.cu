// Launcher of the tile kernels of the MODP ring with 1 E combination per thread
// (one translation unit per E count: these instantiations are the slowest to compile).
#include "tsg_tree_launch.cuh"

namespace tsg {
namespace dev {

tsg_status launch_tile_modp_ne1(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  launch_tile_ring_ne<TSG_RING_MODP, 1>(la, ra, st);
  return TSG_OK;
}

}  // namespace dev
}  // namespace tsg
