// C ABI entry points of the nested likelihood, the outer SMC and the
// stand-alone resampling primitive.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

#define CU(call, where)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return ctx->cuda_fail(e_, where); \
    } while (0)

extern "C" int32_t smcgpu_resample_counts(smcgpu_ctx *ctx, const double *weights, int32_t n, double u0_hi,
                                          double u0_lo, int32_t *counts) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (n < 0 || (n > 0 && (!weights || !counts))) return ctx->fail(SMCGPU_ERR_ARG, "resample: bad arguments");
    if (n == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    CU(ctx->d_w.upload(weights, n, ctx->stream), "upload weights");
    CU(ctx->d_counts.ensure(n), "alloc counts");
    CU(ctx->d_flag.ensure(1), "alloc flag");
    CU(smc::launch_resample_counts(ctx->d_w.p, n, u0_hi, u0_lo, ctx->d_counts.p, ctx->d_flag.p, ctx->stream),
       "resample kernel");
    CU(cudaMemcpyAsync(counts, ctx->d_counts.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
       "copy counts");
    CU(cudaStreamSynchronize(ctx->stream), "sync");
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_fault_likelihood_batch_dev(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                                     uint64_t seed, const uint64_t *streams_dev, double *neglog_dev,
                                                     int32_t *status_dev) {
    (void)n_theta; (void)theta_dev; (void)seed; (void)streams_dev; (void)neglog_dev; (void)status_dev;
    if (!ctx) return SMCGPU_ERR_ARG;
    return ctx->fail(SMCGPU_ERR_STATE, "nested likelihood not available in this build");
}

extern "C" int32_t smcgpu_fault_likelihood_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed,
                                                 const uint64_t *streams, double *neglog_out, int32_t *status_out) {
    (void)n_theta; (void)theta; (void)seed; (void)streams; (void)neglog_out; (void)status_out;
    if (!ctx) return SMCGPU_ERR_ARG;
    return ctx->fail(SMCGPU_ERR_STATE, "nested likelihood not available in this build");
}

extern "C" int32_t smcgpu_fault_smc_exec(smcgpu_ctx *ctx, const double *range, int32_t nparticle, uint64_t seed,
                                         const char *output_dir, double *particles_out, double *likelihood_out,
                                         double *evidence_out, int32_t *nstage_out) {
    (void)range; (void)nparticle; (void)seed; (void)output_dir; (void)particles_out; (void)likelihood_out;
    (void)evidence_out; (void)nstage_out;
    if (!ctx) return SMCGPU_ERR_ARG;
    return ctx->fail(SMCGPU_ERR_STATE, "outer SMC not available in this build");
}
