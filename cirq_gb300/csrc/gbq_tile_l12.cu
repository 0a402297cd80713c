// Tile-pass kernels for 12-bit tiles, single state (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l12(Ctx* c, const PassArgs& a, bool dual) {
  if (dual) return launch_pass_l12_dual(c, a);
  if (pass_kmax(a) == 0) return launch_tile_pass<12, 0, false>(c, a);
  return launch_tile_pass<12, 5, false>(c, a);
}

}  // namespace gbq
