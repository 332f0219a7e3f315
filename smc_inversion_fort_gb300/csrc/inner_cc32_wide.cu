// Inner SMC, MIXED CUDA-core engine, 96- and 128-row tiles (64 < D <= 128);
// the 192-row tile is in inner_cc32_192.cu.
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_cc32_wide(const InnerParts &P, cudaStream_t s, int W) {
    const int D = P.a[0].D;
    if (D <= 96) return launch_cc_t<float, 6>(P, s, W);
    if (D <= 128) return launch_cc_t<float, 8>(P, s, W);
    return launch_inner_cc32_192(P, s, W);
}

}  // namespace smc
