// Tile-pass kernels for 12-bit tiles, two states, with shared-memory dense
// ops (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l12_dual_dense(Ctx* c, const PassArgs& a) { return launch_tile_pass<12, 5, true>(c, a); }

}  // namespace gbq
