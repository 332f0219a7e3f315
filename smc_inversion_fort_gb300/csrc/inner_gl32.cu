// Inner SMC, global-matrix engine in MIXED precision (FP32 stage matrix in
// global memory): D <= 256, 512 and 1024 tiles.
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_gl32(const InnerParts &P, cudaStream_t s) {
    if (P.a[0].D <= 256) return launch_gl_t<float, 16>(P, s);
    if (P.a[0].D <= 512) return launch_gl_t<float, 32>(P, s);
    return launch_gl_t<float, 64>(P, s);
}

}  // namespace smc
