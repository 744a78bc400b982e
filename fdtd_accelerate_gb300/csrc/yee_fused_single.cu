// Single-grid instantiations of the fused kernel (a translation unit of its
// own, compiled in parallel with the host code and the batched ones).
#include "yee_fused.cuh"

namespace fdtd {
namespace fused {

bool single_kernels(int ty, int ns, FusedKernel out[3]) {
#define FDTD_CASE(TY, NS)                                  \
    if (ty == TY && ns == NS) {                            \
        out[0] = k_yee_fused<TY, NS, false, 0>;            \
        out[1] = k_yee_fused<TY, NS, false, 1>;            \
        out[2] = k_yee_fused<TY, NS, false, 2>;            \
        return true;                                       \
    }
    FDTD_FUSED_TILES(FDTD_CASE)
#undef FDTD_CASE
    return false;
}

}  // namespace fused
}  // namespace fdtd
