// Truncated-normal Gibbs initialisation of the inner population
// (slip_gen_init_particles, smc_slip.f90:184-264).
#include "common.cuh"
#include "inner.h"

namespace smc {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace

// One warp per geometry runs the reference's single chained sweep (particle
// k is one sweep after particle k-1, starting at 0).  FP64 uses the
// reference's Newton inverse CDF; MIXED inverts in FP32 through
// normcdff/normcdfinvf on the tail-appropriate side.
template <bool MIXED>
__global__ void gibbs_kernel(MeshDev m, InnerArgs a) {
    extern __shared__ double gsh[];
    const int wpb = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int th = blockIdx.x * wpb + wid;
    if (th >= a.n_theta) return;
    const int D = a.D, N = a.N;
    double *cur = gsh + (size_t)wid * 2 * D, *vn = cur + D;
    const double alpha2 = a.aux[th].alpha2;
    const double *ll = a.llval + (size_t)th * m.ll_nnz;
    const uint64_t stream = a.streams[th];
    double *parts = a.parts + (size_t)th * N * D;
    int stat = 0;
    for (int i = lane; i < D; i += 32) cur[i] = 0.0;
    __syncwarp();
    const double pi = 3.141592653589793;
    for (int k = 0; k < N; ++k) {
        for (int d = lane; d < D; d += 32)
            vn[d] = MIXED ? (double)rng_normal_f(a.seed, stream, RNG_GIBBS, 0, k, d)
                          : rng_normal(a.seed, stream, RNG_GIBBS, 0, k, d);
        __syncwarp();
        for (int i = 0; i < D; ++i) {
            int e0 = m.ll_ptr[i], e1 = m.ll_ptr[i + 1];
            // diagonal entry and the conditional mean
            int e = e0 + lane;
            int j = e < e1 ? m.ll_col[e] : -1;
            double v = e < e1 ? ll[e] : 0.0;
            double s2, mu;
            if (!MIXED) {
                double lii = (j == i) ? v : 0.0, term = 0.0;
                lii = warp_sum(lii);
                s2 = 1.0 / (lii / alpha2);
                if (j >= 0 && j != i) term = v / alpha2 * cur[j] * s2;
                mu = -warp_sum(term);
            } else {
                float lii = (j == i) ? (float)v : 0.0f, term = 0.0f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) lii += __shfl_xor_sync(0xffffffffu, lii, o);
                if (j >= 0 && j != i) term = (float)v * (float)cur[j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
                float s2f = (float)alpha2 / lii;
                s2 = (double)s2f;
                mu = (double)(-term / lii);
            }
            if (lane == 0) {
                double v1 = vn[i];
                double y;
                if (!MIXED) {
                    double sq = sqrt(2.0 * s2), pdfn = sqrt(2.0 * pi * s2);
                    double x = mu + v1 * sqrt(s2);
                    double fx = (1.0 + erf((x - mu) / sq)) / 2.0;
                    double f1 = (1.0 + erf((a.max_slip - mu) / sq)) / 2.0;
                    double f0 = (1.0 + erf((0.0 - mu) / sq)) / 2.0;
                    double target = (f1 - f0) * fx + f0;
                    y = mu;
                    double err = 1.0, yp = y + err;
                    int cnt = 0;
                    while (err > 1e-8 && cnt < 100) {
                        double cdf = (1.0 + erf((y - mu) / sq)) / 2.0;
                        double pdf = exp(-((y - mu) * (y - mu)) / (2.0 * s2)) / pdfn;
                        y = y - (cdf - target) / pdf;
                        err = fabs(y - yp);
                        yp = y;
                        ++cnt;
                    }
                    if (cnt >= 100) stat |= SMCGPU_ST_NEWTON_CAP;
                } else {
                    float sg = sqrtf((float)s2), muf = (float)mu;
                    float al = (0.0f - muf) / sg, be = ((float)a.max_slip - muf) / sg;
                    float u = normcdff((float)v1);
                    float z;
                    if (al >= 0.0f) {
                        float qa = normcdff(-al), qb = normcdff(-be);
                        float q = qa - u * (qa - qb);
                        z = q > 0.0f ? -normcdfinvf(q) : al;
                    } else {
                        float pa = normcdff(al), pb = normcdff(be);
                        float p = pa + u * (pb - pa);
                        z = p > 0.0f ? normcdfinvf(p) : be;
                    }
                    float yf = muf + sg * z;
                    yf = fminf(fmaxf(yf, 0.0f), (float)a.max_slip);
                    y = (double)yf;
                }
                cur[i] = y;
            }
            __syncwarp();
        }
        for (int d = lane; d < D; d += 32) parts[(size_t)k * D + d] = cur[d];
        __syncwarp();
    }
    if (lane == 0 && stat) atomicOr(a.status + th, stat);
}

cudaError_t launch_gibbs(const MeshDev &m, const InnerArgs &a, cudaStream_t s) {
    if (a.n_theta <= 0) return cudaSuccess;
    const int wpb = 4;
    size_t sm = (size_t)wpb * 2 * a.D * sizeof(double);
    unsigned blocks = (unsigned)((a.n_theta + wpb - 1) / wpb);
    if (a.mixed) {
        cudaFuncSetAttribute(gibbs_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        gibbs_kernel<true><<<blocks, wpb * 32, sm, s>>>(m, a);
    } else {
        cudaFuncSetAttribute(gibbs_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        gibbs_kernel<false><<<blocks, wpb * 32, sm, s>>>(m, a);
    }
    return cudaGetLastError();
}

}  // namespace smc
