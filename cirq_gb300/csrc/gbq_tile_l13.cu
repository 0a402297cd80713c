// Tile-pass kernels for 13-bit tiles (see gbq_tile.cuh).
#include "gbq_tile.cuh"

namespace gbq {

int launch_pass_l13(Ctx* c, const PassArgs& a, bool dual) {
  if (dual) {
    set_error("two-state passes support tile widths 10 to 12");
    return GBQ_ERR_ARG;
  }
  if (pass_kmax(a) == 0) return launch_tile_pass<13, 0, false>(c, a);
  return launch_tile_pass<13, 5, false>(c, a);
}

}  // namespace gbq
