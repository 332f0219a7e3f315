// Inner SMC, MIXED CUDA-core engine instantiations up to D = 64; the larger
// row tiles are in their own units (each is a long ptxas job).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_cc32(const InnerParts &P, cudaStream_t s, int W) {
    const int D = P.a[0].D;
    if (D <= 32) return launch_cc_t<float, 2>(P, s, W);
    if (D <= 64) return launch_cc_t<float, 4>(P, s, W);
    return launch_inner_cc32_wide(P, s, W);
}

}  // namespace smc
