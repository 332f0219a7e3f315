// Inner SMC, warp-MMA engine with 8 warps per geometry and two geometries
// per CTA (batches larger than the SM count; D <= 128).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_mma_pair(const InnerParts &P, cudaStream_t s) {
    const int D = P.a[0].D;
    if (D <= 32) return launch_wg_t<2, ENG_MMA, 8>(P, s, 2);
    if (D <= 64) return launch_wg_t<4, ENG_MMA, 8>(P, s, 2);
    return launch_wg_t<8, ENG_MMA, 8>(P, s, 2);
}

}  // namespace smc
