// Launcher of the streaming kernels of the MODP ring (one translation unit per ring and kernel
// family, compiled in parallel).
#include "tsg_tree_launch.cuh"

namespace tsg {
namespace dev {

tsg_status launch_stream_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  return launch_stream_ring<TSG_RING_MODP>(la, ra, st);
}

}  // namespace dev
}  // namespace tsg
