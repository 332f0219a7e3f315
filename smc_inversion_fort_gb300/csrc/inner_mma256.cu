// Inner SMC, warp-MMA engine with the stage matrix streamed from global
// memory (128 < D <= 256), one geometry per CTA of 16 warps.
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_mma_streamed(const InnerParts &P, cudaStream_t s) {
    return launch_wg_t<16, ENG_MMA, 16>(P, s, 1);
}

}  // namespace smc
