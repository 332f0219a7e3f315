// Inner SMC, global-matrix engine in FP64 (the reference's algebra): D <= 256,
// 512 and 1024 tiles.
#include "inner_impl.cuh"

namespace smc {

cudaError_t launch_inner_gl64(const MeshDev &m, const InnerArgs &a, cudaStream_t s) {
    if (a.D <= 256) return launch_gl_t<double, 16>(m, a, s);
    if (a.D <= 512) return launch_gl_t<double, 32>(m, a, s);
    return launch_gl_t<double, 64>(m, a, s);
}

}  // namespace smc
