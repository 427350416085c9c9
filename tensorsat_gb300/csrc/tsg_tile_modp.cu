// Launcher of the tile kernels of the MODP ring: dispatches on the E count to the units
// tsg_tile_modp_ne{1,2,4}.cu, which compile in parallel.
#include "tsg_tree_dev.cuh"

namespace tsg {
namespace dev {

tsg_status launch_tile_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (la.shape.ne) {
    case 1: return launch_tile_modp_ne1(la, ra, st);
    case 2: return launch_tile_modp_ne2(la, ra, st);
    default: return launch_tile_modp_ne4(la, ra, st);
  }
}

}  // namespace dev
}  // namespace tsg
