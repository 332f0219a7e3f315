// Inner SMC, MIXED CUDA-core engine instantiations up to D = 64; the larger
// row tiles are in their own units (each is a long ptxas job).
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_cc32(const MeshDev &m, const InnerArgs &a, cudaStream_t s, int W) {
    const int D = a.D;
    if (D <= 32) return launch_cc_t<float, 2>(m, a, s, W);
    if (D <= 64) return launch_cc_t<float, 4>(m, a, s, W);
    return launch_inner_cc32_wide(m, a, s, W);
}

}  // namespace smc
