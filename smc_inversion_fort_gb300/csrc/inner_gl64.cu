// Inner SMC, global-matrix engine in FP64 (the reference's algebra): D <= 256,
// 512 and 1024 tiles.
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_gl64(const InnerParts &P, cudaStream_t s) {
    if (P.a[0].D <= 256) return launch_gl_t<double, 16>(P, s);
    if (P.a[0].D <= 512) return launch_gl_t<double, 32>(P, s);
    return launch_gl_t<double, 64>(P, s);
}

}  // namespace smc
