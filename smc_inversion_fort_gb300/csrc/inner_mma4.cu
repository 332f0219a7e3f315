// Inner SMC, warp-MMA engine with 4 warps and 16 chain slots per geometry and
// four geometries per CTA (batches of more than two geometries per SM; D <= 64).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_mma_quad(const InnerParts &P, cudaStream_t s) {
    if (P.a[0].D <= 32) return launch_wg_t<2, ENG_MMAQ, 4>(P, s, 4);
    return launch_wg_t<4, ENG_MMAQ, 4>(P, s, 4);
}

}  // namespace smc
