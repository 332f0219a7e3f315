// Inner SMC, warp-MMA engine with 16 warps and one geometry per group
// (batches no larger than the SM count; D <= 128).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_mma_wide(const InnerParts &P, cudaStream_t s) {
    const int D = P.a[0].D;
    if (D <= 32) return launch_wg_t<2, ENG_MMA, 16>(P, s, 1);
    if (D <= 64) return launch_wg_t<4, ENG_MMA, 16>(P, s, 1);
    return launch_wg_t<8, ENG_MMA, 16>(P, s, 1);
}

}  // namespace smc
