// Truncated-normal Gibbs initialisation of the inner population
// (slip_gen_init_particles, smc_slip.f90:184-264).
#include <algorithm>

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

// MIXED: the same sweep in FP32 with the geometry's L^T L rows cached in
// shared memory (off-diagonal columns and values, the diagonal, the
// conditional standard deviation), so that a component update is one
// shared-memory gather per lane, a warp sum and lane 0's inverse CDF.
__global__ void gibbs_mixed_kernel(MeshDev m, InnerArgs a, int maxrow) {
    extern __shared__ __align__(16) unsigned char gsm[];
    const int wpb = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int th = blockIdx.x * wpb + wid;
    if (th >= a.n_theta) return;
    const int D = a.D, N = a.N, D2 = (D + 1) & ~1;
    const size_t per = (size_t)D * maxrow * 8 + (size_t)(2 * D2 + 2 * D) * 4;
    unsigned char *base = gsm + (size_t)wid * ((per + 15) & ~(size_t)15);
    int *rc = (int *)base;                          // [D][maxrow] off-diagonal columns (-1: none)
    float *rv = (float *)(rc + (size_t)D * maxrow); // [D][maxrow] values
    float *cur = rv + (size_t)D * maxrow, *vn = cur + D2, *ilii = vn + D2, *sgr = ilii + D;
    const float alpha2 = (float)a.aux[th].alpha2, mxs = (float)a.max_slip;
    const double *ll = a.llval + (size_t)th * m.ll_nnz;
    const uint64_t stream = a.streams[th];
    double *parts = a.parts + (size_t)th * N * D;
    for (int i = lane; i < D; i += 32) {
        float lii = 0.0f;
        int q = 0;
        for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) {
            const int j = m.ll_col[e];
            if (j == i) {
                lii += (float)ll[e];
            } else {
                rc[(size_t)i * maxrow + q] = j;
                rv[(size_t)i * maxrow + q] = (float)ll[e];
                ++q;
            }
        }
        for (; q < maxrow; ++q) { rc[(size_t)i * maxrow + q] = -1; rv[(size_t)i * maxrow + q] = 0.0f; }
        ilii[i] = 1.0f / lii;
        sgr[i] = sqrtf(alpha2 / lii);
        cur[i] = 0.0f;
    }
    __syncwarp();
    for (int k = 0; k < N; ++k) {
        for (int d2 = lane; d2 < D2 / 2; d2 += 32) {
            const float2 z = rng_normal2_f(a.seed, stream, RNG_GIBBS, 0, (uint64_t)k, (uint64_t)d2);
            vn[2 * d2] = z.x;
            vn[2 * d2 + 1] = z.y;
        }
        __syncwarp();
        for (int i = 0; i < D; ++i) {
            float term = 0.0f;
            if (lane < maxrow) {
                const int j = rc[(size_t)i * maxrow + lane];
                if (j >= 0) term = rv[(size_t)i * maxrow + lane] * cur[j];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
            if (lane == 0) {
                const float muf = -term * ilii[i], sg = sgr[i];
                const float al = (0.0f - muf) / sg, be = (mxs - muf) / sg;
                const float u = normcdff(vn[i]);
                float z;
                if (al >= 0.0f) {
                    const float qa = normcdff(-al), qb = normcdff(-be);
                    const float q = qa - u * (qa - qb);
                    z = q > 0.0f ? -normcdfinvf(q) : al;
                } else {
                    const float pa = normcdff(al), pb = normcdff(be);
                    const float p = pa + u * (pb - pa);
                    z = p > 0.0f ? normcdfinvf(p) : be;
                }
                cur[i] = fminf(fmaxf(muf + sg * z, 0.0f), mxs);
            }
            __syncwarp();
        }
        for (int d = lane; d < D; d += 32) parts[(size_t)k * D + d] = (double)cur[d];
        __syncwarp();
    }
}

cudaError_t launch_gibbs(const MeshDev &m, const InnerArgs &a, cudaStream_t s) {
    if (a.n_theta <= 0) return cudaSuccess;
    const int wpb = 4;
    size_t sm = (size_t)wpb * 2 * a.D * sizeof(double);
    unsigned blocks = (unsigned)((a.n_theta + wpb - 1) / wpb);
    if (a.mixed) {
        // one warp per geometry; as many per block as shared memory allows (4 at most)
        const int maxrow = m.ll_maxrow;   // at most 32: one entry per lane
        const int D2 = (a.D + 1) & ~1;
        const size_t per = (((size_t)a.D * maxrow * 8 + (size_t)(2 * D2 + 2 * a.D) * 4) + 15) & ~(size_t)15;
        int dev = 0, maxsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        const int w = (int)std::max<size_t>(1, std::min<size_t>(4, (size_t)maxsm / per));
        const size_t smm = per * w;
        cudaError_t e = cudaFuncSetAttribute(gibbs_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smm);
        if (e != cudaSuccess) return e;
        gibbs_mixed_kernel<<<(unsigned)((a.n_theta + w - 1) / w), w * 32, smm, s>>>(m, a, maxrow);
    } else {
        cudaFuncSetAttribute(gibbs_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        gibbs_kernel<false><<<blocks, wpb * 32, sm, s>>>(m, a);
    }
    return cudaGetLastError();
}

}  // namespace smc
