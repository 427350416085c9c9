// Launcher of the packed-step kernel (the small steps of one tree level, of several
// instances, in one launch), in its own translation unit.
#include "tsg_tree_dev.cuh"

namespace tsg {
namespace dev {

tsg_status launch_pack(int ring, const PackArgs& a, const RingArgs& ra, cudaStream_t st) {
  if (a.n_items <= 0 || a.n_warps == 0) return TSG_OK;
  const unsigned blocks = (a.n_warps + (kThreads / 32) - 1) / (kThreads / 32);
  switch (ring) {
    case TSG_RING_OR_AND:
      tree_pack_kernel<TSG_RING_OR_AND><<<blocks, kThreads, 0, st>>>(a, ra);
      break;
    case TSG_RING_U64:
      tree_pack_kernel<TSG_RING_U64><<<blocks, kThreads, 0, st>>>(a, ra);
      break;
    default:
      tree_pack_kernel<TSG_RING_MODP><<<blocks, kThreads, 0, st>>>(a, ra);
      break;
  }
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

}  // namespace dev
}  // namespace tsg
