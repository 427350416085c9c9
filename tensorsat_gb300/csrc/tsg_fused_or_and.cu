// Launcher of the fused tree-step kernels of the OR-AND ring (one translation unit per
// ring, compiled in parallel with the others).
#include "tsg_tree_launch.cuh"

namespace tsg {
namespace dev {

tsg_status launch_fused_or_and(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  return launch_fused_ring<TSG_RING_OR_AND>(la, ra, st);
}

}  // namespace dev
}  // namespace tsg
