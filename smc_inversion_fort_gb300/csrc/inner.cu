// Inner tempered SMC over slip (slip_smc_exec, smc_slip.f90:1445-1663):
// engine and configuration choice.  The kernel and launcher templates are in
// inner_impl.cuh; each inner_*.cu unit instantiates one family of them.
#include <cuda_runtime.h>

#include "inner.h"

namespace smc {

// Which engine runs a batch (shared with the driver's buffer sizing).
bool inner_uses_global(int mixed, int engine, int D) {
    if (engine == SMCGPU_ENGINE_GLOBAL) return true;
    if (!mixed) return D > 128;
    if (engine == SMCGPU_ENGINE_MMA) return D > 256;
    if (engine == SMCGPU_ENGINE_TCGEN05) return D > 192;   // tcgen05 hands 128 < D <= 192 to the CUDA cores
    return D > 192;
}

const char *inner_size_limit(int mixed, int engine, int D, int N) {
    if (N > 32767) return "nparticle_slip must be < 32768";
    if (D > 1024) return mixed ? "slip dimension too large for the MIXED inner kernel (D <= 1024)"
                               : "slip dimension too large for the FP64 inner kernel (D <= 1024)";
    (void)engine;
    return nullptr;
}

cudaError_t launch_inner(const MeshDev &m, const InnerArgs &a, cudaStream_t s, const char **why) {
    if (a.n_theta <= 0) return cudaSuccess;
    if (a.N > 32767) { *why = "nparticle_slip must be < 32768"; return cudaErrorInvalidValue; }
    const int D = a.D;
    const int W = a.warps_per_theta;
    if (inner_uses_global(a.mixed, a.engine, D)) {
        if (!a.mgl || !a.glxc) { *why = "inner kernel: global stage-matrix buffers missing"; return cudaErrorInvalidValue; }
        if (!a.mixed) {
            if (D <= 1024) return launch_inner_gl64(m, a, s);
            *why = "slip dimension too large for the FP64 inner kernel (D <= 1024)";
            return cudaErrorInvalidValue;
        }
        if (D <= 1024) return launch_inner_gl32(m, a, s);
        *why = "slip dimension too large for the MIXED inner kernel (D <= 1024)";
        return cudaErrorInvalidValue;
    }
    if (!a.mixed) return launch_inner_fp64(m, a, s, W);
    if (a.engine == SMCGPU_ENGINE_MMA && D > 128) {
        // stage matrix streamed from global memory, one geometry per CTA of 16 warps
        if (!a.afrag || !a.A32) { *why = "inner kernel: stage-matrix buffers missing"; return cudaErrorInvalidValue; }
        return launch_inner_mma_streamed(m, a, s);
    } else if (a.engine == SMCGPU_ENGINE_MMA) {
        // 16 warps per geometry while the batch leaves SMs free (lowest
        // latency per geometry), 8 warps and two geometries per CTA beyond
        int nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        return a.n_theta <= nsm ? launch_inner_mma_wide(m, a, s) : launch_inner_mma_pair(m, a, s);
    } else if (a.engine == SMCGPU_ENGINE_TCGEN05 && D <= 128) {
        return launch_inner_tc(m, a, s);
    }
    return launch_inner_cc32(m, a, s, W);
}

}  // namespace smc
