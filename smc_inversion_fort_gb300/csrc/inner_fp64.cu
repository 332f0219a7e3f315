// Inner SMC, FP64 CUDA-core engine instantiations up to D = 64; the 96- and
// 128-row tiles are in their own units (each is a long ptxas job).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_fp64(const InnerParts &P, cudaStream_t s, int W) {
    const int D = P.a[0].D;
    if (D <= 32) return launch_cc_t<double, 2>(P, s, W);
    if (D <= 64) return launch_cc_t<double, 4>(P, s, W);
    if (D <= 96) return launch_inner_fp64_96(P, s, W);
    return launch_inner_fp64_128(P, s, W);
}

}  // namespace smc
