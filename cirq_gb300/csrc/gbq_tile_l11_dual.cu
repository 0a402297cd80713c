// Tile-pass kernels for 11-bit tiles, two states (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l11_dual(Ctx* c, const PassArgs& a) {
  if (pass_kmax(a) == 0) return launch_tile_pass<11, 0, true>(c, a);
  return launch_tile_pass<11, 5, true>(c, a);
}

}  // namespace gbq
