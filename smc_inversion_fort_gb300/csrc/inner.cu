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

long long inner_launch_key(int mixed, int engine, int D, int warps, int n_total) {
    // family: 1 GL32, 2 GL64, 3 FP64 CUDA cores, 4 MMA streamed, 5 MMA wide,
    // 6 MMA pair, 7 tcgen05, 8 FP32 CUDA cores, 9 MMA quad; row tile as the
    // families pick it
    int fam, rt;
    if (inner_uses_global(mixed, engine, D)) {
        fam = mixed ? 1 : 2;
        rt = D <= 256 ? 16 : D <= 512 ? 32 : 64;
    } else if (!mixed) {
        fam = 3;
        rt = D <= 32 ? 2 : D <= 64 ? 4 : D <= 96 ? 6 : 8;
    } else if (engine == SMCGPU_ENGINE_MMA && D > 128) {
        fam = 4;
        rt = 16;
    } else if (engine == SMCGPU_ENGINE_MMA) {
        int nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        fam = n_total <= nsm ? 5 : (D <= 64 && n_total > 2 * nsm) ? 9 : 6;
        rt = D <= 32 ? 2 : D <= 64 ? 4 : 8;
    } else if (engine == SMCGPU_ENGINE_TCGEN05 && D <= 128) {
        fam = 7;
        rt = D <= 32 ? 2 : D <= 64 ? 4 : 8;
    } else {
        fam = 8;
        rt = D <= 32 ? 2 : D <= 64 ? 4 : D <= 96 ? 6 : D <= 128 ? 8 : 12;
    }
    const int w = (fam == 3 || fam == 8) ? warps : 0;
    return ((long long)fam * 1000 + rt) * 1000 + w;
}

cudaError_t launch_inner(const MeshDev &m, const InnerArgs &a, cudaStream_t s, const char **why) {
    if (a.n_theta <= 0) return cudaSuccess;
    InnerParts P;
    P.n = 1;
    P.start[0] = 0;
    P.start[1] = a.n_theta;
    P.m[0] = m;
    P.a[0] = a;
    return launch_inner_parts(P, s, why);
}

cudaError_t launch_inner_parts(const InnerParts &P, cudaStream_t s, const char **why) {
    if (P.n <= 0 || P.n > INNER_MAX_PARTS) { *why = "inner kernel: bad part count"; return cudaErrorInvalidValue; }
    const int ntot = P.start[P.n];
    if (ntot <= 0) return cudaSuccess;
    const InnerArgs &a = P.a[0];
    const int D = a.D;
    const int W = a.warps_per_theta;
    const long long key = inner_launch_key(a.mixed, a.engine, D, W, ntot);
    for (int p = 0; p < P.n; ++p) {
        const InnerArgs &ap = P.a[p];
        if (ap.N > 32767) { *why = "nparticle_slip must be < 32768"; return cudaErrorInvalidValue; }
        if (P.start[p + 1] - P.start[p] != ap.n_theta || ap.mixed != a.mixed ||
            inner_launch_key(ap.mixed, ap.engine, ap.D, ap.warps_per_theta, ntot) != key) {
            *why = "inner kernel: the parts of one launch must share the kernel configuration";
            return cudaErrorInvalidValue;
        }
    }
    if (inner_uses_global(a.mixed, a.engine, D)) {
        for (int p = 0; p < P.n; ++p)
            if (!P.a[p].mgl || !P.a[p].glxc) { *why = "inner kernel: global stage-matrix buffers missing"; return cudaErrorInvalidValue; }
        if (!a.mixed) {
            if (D <= 1024) return launch_inner_gl64(P, s);
            *why = "slip dimension too large for the FP64 inner kernel (D <= 1024)";
            return cudaErrorInvalidValue;
        }
        if (D <= 1024) return launch_inner_gl32(P, s);
        *why = "slip dimension too large for the MIXED inner kernel (D <= 1024)";
        return cudaErrorInvalidValue;
    }
    if (!a.mixed) return launch_inner_fp64(P, s, W);
    if (a.engine == SMCGPU_ENGINE_MMA && D > 128) {
        // stage matrix streamed from global memory, one geometry per CTA of 16 warps
        for (int p = 0; p < P.n; ++p)
            if (!P.a[p].afrag || !P.a[p].A32) { *why = "inner kernel: stage-matrix buffers missing"; return cudaErrorInvalidValue; }
        return launch_inner_mma_streamed(P, s);
    } else if (a.engine == SMCGPU_ENGINE_MMA) {
        // 16 warps per geometry while the batch leaves SMs free (lowest
        // latency per geometry), 8 warps and two geometries per CTA up to two
        // geometries per SM; beyond, up to 64 slip dimensions, 4 warps and 16
        // chain slots per geometry and four geometries per CTA (more geometries
        // in flight per SM: the step chain is latency-bound, and the slots of a
        // geometry are half idle anyway, the rounds of a stage being set by its
        // longest Metropolis chain)
        int nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (ntot <= nsm) return launch_inner_mma_wide(P, s);
        if (D <= 64 && ntot > 2 * nsm) return launch_inner_mma_quad(P, s);
        return launch_inner_mma_pair(P, s);
    } else if (a.engine == SMCGPU_ENGINE_TCGEN05 && D <= 128) {
        return launch_inner_tc(P, s);
    }
    return launch_inner_cc32(P, s, W);
}

}  // namespace smc
