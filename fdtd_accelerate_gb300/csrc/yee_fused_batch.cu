// Batched instantiations of the fused kernel (many grids per launch; the z
// slab on the batched band kernels).
#include "yee_fused.cuh"

namespace fdtd {
namespace fused {

bool batch_kernels(int ty, int ns, FusedKernel out[2]) {
#define FDTD_CASE(TY, NS)                                  \
    if (ty == TY && ns == NS) {                            \
        out[0] = k_yee_fused<TY, NS, true, 0>;          \
        out[1] = k_yee_fused<TY, NS, true, 1>;          \
        return true;                                       \
    }
    FDTD_FUSED_TILES(FDTD_CASE)
#undef FDTD_CASE
    return false;
}

}  // namespace fused
}  // namespace fdtd
