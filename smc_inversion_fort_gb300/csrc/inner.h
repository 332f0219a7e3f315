// Inner tempered SMC over slip (slip_smc_exec, smc_slip.f90:1445-1663):
// per-batch argument block and launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "mesh.h"

namespace smc {

struct InnerArgs {
    int n_theta, N, NP2, D, mixed;
    int ntau, tf, max_stages;
    int warps_per_theta;  // CUDA-core engine: warps per geometry (1, 2, 4, 8; 0 picks by batch size)
    int engine;           // step engine, SMCGPU_ENGINE_* (warp MMA: D <= 256, tcgen05: D <= 128, global: any)
    double cv, max_slip;
    uint64_t seed;
    const unsigned long long *streams;  // [n_theta]
    // per-theta operator data
    const double *A;      // [th][D][D] column-major Gram matrix
    float *A32;           // [th][D][D] FP32 copy (MIXED), written by the inner kernel
    float *lv32;          // [th][nrow][9] FP32 copy of the L values (MIXED), written by the inner kernel
    float *ll32;          // [th][ll_nnz] FP32 copy of the L^T L values (MIXED), written by the inner kernel
    uint4 *afrag;         // [th][256 * 256 / 4] stage matrix in MMA-fragment order (MIXED, 128 < D <= 256)
    void *mgl;            // global-matrix engine: [th][D][D] stage matrix (float MIXED, double FP64)
    void *glxc;           // global-matrix engine: [th][16][D] chain states of the slots (same type; 8 slots
                          // in FP64 beyond 512 dimensions)
    int *queue;           // device counter of the persistent launch (nullptr: one CTA per G geometries)
    const double *b;      // [th][D]
    const double *dsd;    // [th]
    const double *lval;   // [th][nrow][9] values of L (columns in MeshDev::l_col)
    const double *llval;  // [th][ll_nnz] values of L^T L on MeshDev::ll_ptr/ll_col
    const ThetaAux *aux;  // [th]
    // per-theta state (N = inner particles, NP2 = next power of two >= N)
    double *parts, *parts_new;   // [th][N][D]
    double *dbuf;                // [th][9][N]: L, P, Lnew, Pnew, w, dtau, dtau_new, score, spare
    int *ibuf;                   // [th][4][NP2]: assigned, id_start, parent_of / queue keys, subset
    // outputs
    double *neglog;              // [th]
    int *status;                 // [th]
    int *nstage;                 // [th]
    double *trace_gamma;         // optional [th][max_stages+2]
    double *trace_inc;           // optional [th][max_stages+2]
    unsigned long long *counters;  // optional: [0] += tempering stages, [1] += HMC trajectories
};

// One inner launch over several parts of a batch: the per-mesh parts of a
// batch whose geometries carry different meshes (each part with its own mesh
// tables and buffers).  Part p's geometries are the launch's queue indices
// start[p] .. start[p+1]-1 (start[0] = 0); the launch takes its configuration
// and its queue counter from part 0, and every part must map to the same
// kernel instantiation (inner_launch_key).  A single batch is one part.
constexpr int INNER_MAX_PARTS = 24;   // keeps the by-value kernel parameters under 32 KB
struct InnerParts {
    int n = 0;
    int start[INNER_MAX_PARTS + 1] = {0};
    MeshDev m[INNER_MAX_PARTS];
    InnerArgs a[INNER_MAX_PARTS];
};

cudaError_t launch_gibbs(const MeshDev &m, const InnerArgs &a, cudaStream_t s);
// true when a batch of this precision / engine / slip dimension runs on the
// global-matrix engine (InnerArgs::mgl and ::glxc must then be set)
bool inner_uses_global(int mixed, int engine, int D);
// message when no inner engine takes this slip dimension / particle count (else nullptr)
const char *inner_size_limit(int mixed, int engine, int D, int N);
cudaError_t launch_inner(const MeshDev &m, const InnerArgs &a, cudaStream_t s, const char **why);
cudaError_t launch_inner_parts(const InnerParts &P, cudaStream_t s, const char **why);
// The kernel instantiation (engine family, row tile, warps per geometry) that
// runs a part of this precision / engine / slip dimension in a launch of
// n_total geometries: parts with equal keys can share one launch.
long long inner_launch_key(int mixed, int engine, int D, int warps, int n_total);

// engine families behind launch_inner, one translation unit each; the slip
// dimension of part 0 picks the row tile (all parts share it)
cudaError_t launch_inner_fp64(const InnerParts &P, cudaStream_t s, int W);           // D <= 128
cudaError_t launch_inner_fp64_96(const InnerParts &P, cudaStream_t s, int W);        // 64 < D <= 96
cudaError_t launch_inner_fp64_128(const InnerParts &P, cudaStream_t s, int W);       // 96 < D <= 128
cudaError_t launch_inner_cc32(const InnerParts &P, cudaStream_t s, int W);           // D <= 192
cudaError_t launch_inner_cc32_wide(const InnerParts &P, cudaStream_t s, int W);      // 64 < D <= 192
cudaError_t launch_inner_cc32_192(const InnerParts &P, cudaStream_t s, int W);       // 128 < D <= 192
cudaError_t launch_inner_mma_wide(const InnerParts &P, cudaStream_t s);              // D <= 128
cudaError_t launch_inner_mma_pair(const InnerParts &P, cudaStream_t s);              // D <= 128
cudaError_t launch_inner_mma_quad(const InnerParts &P, cudaStream_t s);              // D <= 64
cudaError_t launch_inner_mma_streamed(const InnerParts &P, cudaStream_t s);          // 128 < D <= 256
cudaError_t launch_inner_tc(const InnerParts &P, cudaStream_t s);                    // D <= 128
cudaError_t launch_inner_gl32(const InnerParts &P, cudaStream_t s);                  // D <= 1024
cudaError_t launch_inner_gl64(const InnerParts &P, cudaStream_t s);                  // D <= 1024

}  // namespace smc
