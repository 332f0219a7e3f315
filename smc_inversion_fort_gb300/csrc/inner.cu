// Inner tempered SMC over slip (slip_smc_exec, smc_slip.f90:1445-1663):
// engine and configuration choice.  The kernel and launcher templates are in
// inner_impl.cuh; each inner_*.cu unit instantiates one family of them.
#include <cuda_runtime.h>

#include "inner.h"

namespace smc {

cudaError_t launch_inner(const MeshDev &m, const InnerArgs &a, cudaStream_t s, const char **why) {
    if (a.n_theta <= 0) return cudaSuccess;
    if (a.N > 32767) { *why = "nparticle_slip must be < 32768"; return cudaErrorInvalidValue; }
    const int D = a.D;
    const int W = a.warps_per_theta;
    if (!a.mixed) {
        if (D <= 128) return launch_inner_fp64(m, a, s, W);
        *why = "slip dimension too large for the FP64 inner kernel (D <= 128)";
        return cudaErrorInvalidValue;
    } else if (a.engine == SMCGPU_ENGINE_MMA && D > 128 && D <= 256) {
        // stage matrix streamed from global memory, one geometry per CTA of 16 warps
        if (!a.afrag || !a.A32) { *why = "inner kernel: stage-matrix buffers missing"; return cudaErrorInvalidValue; }
        return launch_inner_mma_streamed(m, a, s);
    } else if (a.engine == SMCGPU_ENGINE_MMA && D <= 128) {
        // 16 warps per geometry while the batch leaves SMs free (lowest
        // latency per geometry), 8 warps and two geometries per CTA beyond
        int nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        return a.n_theta <= nsm ? launch_inner_mma_wide(m, a, s) : launch_inner_mma_pair(m, a, s);
    } else if (a.engine == SMCGPU_ENGINE_TCGEN05 && D <= 128) {
        return launch_inner_tc(m, a, s);
    } else if (D <= 192) {
        return launch_inner_cc32(m, a, s, W);
    }
    *why = "slip dimension too large for the MIXED inner kernel (warp MMA: D <= 256, CUDA cores: D <= 192, "
           "tcgen05: D <= 128)";
    return cudaErrorInvalidValue;
}

}  // namespace smc
