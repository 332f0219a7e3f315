// Inner SMC, FP64 CUDA-core engine, 128-row tile (96 < D <= 128).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_fp64_128(const InnerParts &P, cudaStream_t s, int W) {
    return launch_cc_t<double, 8>(P, s, W);
}

}  // namespace smc
