// Truncated-normal Gibbs initialisation of the inner population
// (slip_gen_init_particles, smc_slip.f90:184-264).
#include <algorithm>

#include "common.cuh"
#include "inner.h"

namespace smc {

// One warp per geometry runs the reference's single chained sweep (particle
// k is one sweep after particle k-1, starting at 0).  The sweep goes level by
// level (MeshDev::gb_order): the components of a level are not coupled, so
// the lanes update them together and the result equals the sequential sweep.
// Each lane follows the reference's arithmetic for its component (the
// conditional mean summed over j != i in ascending j, no contractions) and its
// Newton inverse CDF.
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
        for (int d = lane; d < D; d += 32) vn[d] = rng_normal(a.seed, stream, RNG_GIBBS, 0, k, d);
        __syncwarp();
        for (int lv = 0; lv < m.gb_nlevel; ++lv) {
            const int q1 = m.gb_lvl_ptr[lv + 1];
            for (int q = m.gb_lvl_ptr[lv] + lane; q < q1; q += 32) {
                const int i = m.gb_order[q];
                const int e0 = m.ll_ptr[i], e1 = m.ll_ptr[i + 1];
                double lii = 0.0;
                for (int e = e0; e < e1; ++e)
                    if (m.ll_col[e] == i) lii = ll[e];
                const double s2 = 1.0 / (lii / alpha2);
                double mu = 0.0;
                for (int e = e0; e < e1; ++e) {
                    const int j = m.ll_col[e];
                    if (j != i) mu = __dsub_rn(mu, __dmul_rn(__dmul_rn(ll[e] / alpha2, cur[j]), s2));
                }
                const double v1 = vn[i];
                const double sq = sqrt(2.0 * s2), pdfn = sqrt(2.0 * pi * s2);
                const double x = __dadd_rn(mu, __dmul_rn(v1, sqrt(s2)));
                const double fx = (1.0 + erf((x - mu) / sq)) / 2.0;
                const double f1 = (1.0 + erf((a.max_slip - mu) / sq)) / 2.0;
                const double f0 = (1.0 + erf((0.0 - mu) / sq)) / 2.0;
                const double target = __dadd_rn(__dmul_rn(f1 - f0, fx), f0);
                double y = mu, err = 1.0, yp = y + err;
                int cnt = 0;
                while (err > 1e-8 && cnt < 100) {
                    const double cdf = (1.0 + erf((y - mu) / sq)) / 2.0;
                    const double pdf = exp(-__dmul_rn(y - mu, y - mu) / (2.0 * s2)) / pdfn;
                    y = y - (cdf - target) / pdf;
                    err = fabs(y - yp);
                    yp = y;
                    ++cnt;
                }
                if (cnt >= 100) stat |= SMCGPU_ST_NEWTON_CAP;
                cur[i] = y;
            }
            __syncwarp();
        }
        for (int d = lane; d < D; d += 32) parts[(size_t)k * D + d] = cur[d];
        __syncwarp();
    }
    stat = __reduce_or_sync(0xffffffffu, stat);
    if (lane == 0 && stat) atomicOr(a.status + th, stat);
}

// MIXED: the same level-by-level sweep in FP32 with the geometry's L^T L
// rows cached in shared memory (off-diagonal columns and values, the
// diagonal, the conditional standard deviation): a component update is one
// lane's row sum out of shared memory and its FP32 inverse CDF.
__global__ void gibbs_mixed_kernel(MeshDev m, InnerArgs a, int maxrow) {
    extern __shared__ __align__(16) unsigned char gsm[];
    const int wpb = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int th = blockIdx.x * wpb + wid;
    const int D = a.D, N = a.N, D2 = (D + 1) & ~1;
    const size_t per = (size_t)D * maxrow * 8 + (size_t)(2 * D2 + 2 * D) * 4;
    unsigned char *base = gsm + (size_t)wid * ((per + 15) & ~(size_t)15);
    // the sweep's level tables, shared by the block's warps (loaded by every
    // thread of the block before any warp leaves)
    int *ord = (int *)(gsm + (size_t)wpb * ((per + 15) & ~(size_t)15)), *lvl = ord + D;
    for (int q = threadIdx.x; q < D; q += blockDim.x) ord[q] = m.gb_order[q];
    for (int q = threadIdx.x; q <= m.gb_nlevel; q += blockDim.x) lvl[q] = m.gb_lvl_ptr[q];
    __syncthreads();
    if (th >= a.n_theta) return;
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
        // level by level, one component per lane (see gibbs_kernel); the row
        // sum runs without branches (padding entries add an exact zero) so
        // that its loads can be issued ahead of the FMA chain
        for (int lv = 0; lv < m.gb_nlevel; ++lv) {
            const int q1 = lvl[lv + 1];
            for (int q = lvl[lv] + lane; q < q1; q += 32) {
                const int i = ord[q];
                const int *ri = rc + (size_t)i * maxrow;
                const float *vi = rv + (size_t)i * maxrow;
                float term = 0.0f;
#pragma unroll 4
                for (int r = 0; r < maxrow; ++r) {
                    const int j = ri[r];
                    term = fmaf(vi[r], j >= 0 ? cur[j] : 0.0f, term);
                }
                const float muf = -term * ilii[i], sg = sgr[i];
                const float al = (0.0f - muf) / sg, be = (mxs - muf) / sg;
                const float u = normcdff(vn[i]);
                float z;
                if (al >= 0.0f) {
                    const float qa = normcdff(-al), qb = normcdff(-be);
                    const float qq = qa - u * (qa - qb);
                    z = qq > 0.0f ? -normcdfinvf(qq) : al;
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
        const size_t tables = (size_t)(a.D + m.gb_nlevel + 1) * sizeof(int);
        const int w = (int)std::max<size_t>(1, std::min<size_t>(4, ((size_t)maxsm - tables) / per));
        const size_t smm = per * w + tables;
        cudaError_t e = cudaFuncSetAttribute(gibbs_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smm);
        if (e != cudaSuccess) return e;
        gibbs_mixed_kernel<<<(unsigned)((a.n_theta + w - 1) / w), w * 32, smm, s>>>(m, a, maxrow);
    } else {
        cudaFuncSetAttribute(gibbs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        gibbs_kernel<<<blocks, wpb * 32, sm, s>>>(m, a);
    }
    return cudaGetLastError();
}

}  // namespace smc
