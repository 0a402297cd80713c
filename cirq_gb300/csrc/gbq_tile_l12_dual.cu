// Tile-pass kernels for 12-bit tiles, two states, register and diagonal ops
// only (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l12_dual(Ctx* c, const PassArgs& a) {
  if (pass_kmax(a) == 0) return launch_tile_pass<12, 0, true>(c, a);
  return launch_pass_l12_dual_dense(c, a);
}

}  // namespace gbq
