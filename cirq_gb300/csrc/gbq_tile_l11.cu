// Tile-pass kernels for 11-bit tiles (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l11(Ctx* c, const PassArgs& a, bool dual) {
  if (dual) {
    if (pass_kmax(a) == 0) return launch_tile_pass<11, 0, true>(c, a);
    return launch_tile_pass<11, 5, true>(c, a);
  }
  if (pass_kmax(a) == 0) return launch_tile_pass<11, 0, false>(c, a);
  return launch_tile_pass<11, 5, false>(c, a);
}

}  // namespace gbq
