// Launcher of the streaming kernels of the U64 ring (one translation unit per ring and kernel
// family, compiled in parallel).
#include "tsg_tree_launch.cuh"

namespace tsg {
namespace dev {

tsg_status launch_stream_u64(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  return launch_stream_ring<TSG_RING_U64>(la, ra, st);
}

}  // namespace dev
}  // namespace tsg
