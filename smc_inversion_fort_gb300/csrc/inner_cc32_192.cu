// Inner SMC, MIXED CUDA-core engine, 192-row tile (128 < D <= 192).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_cc32_192(const InnerParts &P, cudaStream_t s, int W) {
    return launch_cc_t<float, 12>(P, s, W);
}

}  // namespace smc
