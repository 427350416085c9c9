// Launcher of the fused streaming kernels of the MODP ring (one translation unit per
// ring, compiled in parallel with the others).
#include "tsg_tree_launch.cuh"

namespace tsg {
namespace dev {

tsg_status launch_stream_fused_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  return launch_stream_fused_ring<TSG_RING_MODP>(la, ra, st);
}

}  // namespace dev
}  // namespace tsg
