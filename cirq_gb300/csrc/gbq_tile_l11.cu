// Tile-pass kernels for 11-bit tiles, single state (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l11(Ctx* c, const PassArgs& a, bool dual) {
  if (dual) return launch_pass_l11_dual(c, a);
  if (pass_kmax(a) == 0) return launch_tile_pass<11, 0, false>(c, a);
  return launch_tile_pass<11, 5, false>(c, a);
}

}  // namespace gbq
