// Inner SMC, FP64 CUDA-core engine, 96-row tile (64 < D <= 96).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_fp64_96(const InnerParts &P, cudaStream_t s, int W) {
    return launch_cc_t<double, 6>(P, s, W);
}

}  // namespace smc
