// Green's-function build that allocates nothing on the call path.
//
// smcgpu_greens_batch_dev needs a per-call scratch buffer for the per-plane
// geometry records that the plane kernel writes and the Green's kernel
// reads, and grows it with cudaMalloc when a batch is larger than any seen
// before.  Some callers cannot allocate device memory at that point: a host
// application that hands all of the GPU's memory to its own pool allocator
// at start-up (a later cudaMalloc then fails or fragments the pool), or a
// stage loop that must not take cudaMalloc / cudaFree's device-wide
// synchronisation between its launches.  For them this variant keeps the
// scratch in a fixed file-scope device array instead.
//
// Limits and rules:
//  * at most SMCGPU_NOALLOC_MAX_PLANE_RECORDS plane records per call, i.e.
//    n_theta * nplane <= 16384 (16384 records of 136 bytes, 2.2 MB, held by
//    every GPU that loads the library until the process exits);
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture.  The address is cached per device index for
//    the life of the process, so it goes stale if the device's primary
//    context is destroyed (cudaDeviceReset): no call may follow a reset;
//  * every call shares the one array and it keeps the last call's records:
//    calls whose launches overlap on the GPU race on it, so calls on one
//    device must be ordered (same stream, or synchronised);
//  * no cudaMalloc, cudaFree or allocating library routine is called.  The
//    observation tables it reads were placed on the device by
//    smcgpu_set_data when the context was set up.
#include <mutex>

#include "context.h"

#define SMCGPU_NOALLOC_MAX_PLANE_RECORDS 16384

namespace {

static __device__ __align__(256) smc::PlaneGeom g_noalloc_planes[SMCGPU_NOALLOC_MAX_PLANE_RECORDS];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
smc::PlaneGeom *g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_planes on the current device (looked up once).
cudaError_t noalloc_planes_address(int device, smc::PlaneGeom **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_planes);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[device] = (smc::PlaneGeom *)p;
    }
    *out = g_noalloc_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int32_t smcgpu_greens_batch_noalloc(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                               int32_t precision, void *gmat_dev) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!ctx->has_data) return ctx->fail(SMCGPU_ERR_NODATA, "greens_noalloc: set_data not called");
    if (n_theta < 0 || (n_theta > 0 && (!theta_dev || !gmat_dev)))
        return ctx->fail(SMCGPU_ERR_ARG, "greens_noalloc: bad arguments");
    if (precision != SMCGPU_PREC_FP64 && precision != SMCGPU_PREC_FP32)
        return ctx->fail(SMCGPU_ERR_ARG, "greens_noalloc: precision must be FP64 or FP32");
    if ((long long)n_theta * ctx->mesh.nplane > SMCGPU_NOALLOC_MAX_PLANE_RECORDS)
        return ctx->fail(SMCGPU_ERR_ARG, "greens_noalloc: n_theta * nplane exceeds the fixed scratch of "
                                         "16384 plane records; split the batch");
    if (n_theta == 0) return SMCGPU_OK;
    cudaError_t e = cudaSetDevice(ctx->cfg.device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    smc::PlaneGeom *planes = nullptr;
    e = noalloc_planes_address(ctx->cfg.device, &planes);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaGetSymbolAddress");
    e = smc::launch_planes(ctx->md, n_theta, theta_dev, planes, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "planes kernel");
    e = smc::launch_greens(ctx->md, n_theta, planes, precision, gmat_dev, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "greens kernel");
    return SMCGPU_OK;
}
