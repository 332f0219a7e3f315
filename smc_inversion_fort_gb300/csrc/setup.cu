// Per-theta prior setup: values of the smoothing operator L and of L^T on
// the fixed pattern (gen_laplacian + gen_sparse_lmat, init.f90:295-521),
// L^T L on its structural pattern (calc_ll, init.f90:523-541) and the
// hyper-parameters of get_sigma (init.f90:175-196) / fault_calc_likelihood
// (smc_fault.f90:146-173).
//
// Every entry of L is k * t with k a small integer and t one of
// 1/dxi^2, 1/deta^2, 1/(4 dxi deta) of its plane; the reference accumulates
// the same terms one at a time, which yields exactly k * t, so the values
// here are bit-identical to the reference's.
#include "common.cuh"
#include "kernels.h"
#include "mesh.h"

namespace smc {

__device__ __forceinline__ double stencil_value(const signed char *k, const PlaneGeom &g) {
    double tx = 1.0 / (g.dxi * g.dxi), ty = 1.0 / (g.deta * g.deta), tc = 1.0 / (4.0 * g.dxi * g.deta);
    return (double)k[0] * tx + (double)k[1] * ty + (double)k[2] * tc;
}

__global__ void setup_kernel(MeshDev m, int n_theta, const double *__restrict__ theta,
                             const PlaneGeom *__restrict__ planes, double *__restrict__ lval,
                             double *__restrict__ ltval, double *__restrict__ llval, ThetaAux *__restrict__ aux) {
    const int per = m.nrow + m.D + m.D + 1;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_theta * per) return;
    int th = (int)(t / per), it = (int)(t % per);
    const PlaneGeom *pg = planes + (size_t)th * m.nplane;
    if (it < m.nrow) {
        int r = it;
        const PlaneGeom g = pg[m.l_plane[r]];
        double *out = lval + ((size_t)th * m.nrow + r) * 9;
        for (int q = 0; q < 9; ++q) {
            int c = m.l_col[r * 9 + q];
            out[q] = c >= 0 ? stencil_value(m.l_k + (r * 9 + q) * 3, g) : 0.0;
        }
        return;
    }
    it -= m.nrow;
    if (it < m.D) {
        int c = it;
        const PlaneGeom g = pg[m.lt_plane[c]];
        double *out = ltval + ((size_t)th * m.D + c) * 9;
        for (int q = 0; q < 9; ++q) {
            int r = m.lt_row[c * 9 + q];
            out[q] = r >= 0 ? stencil_value(m.lt_k + (c * 9 + q) * 3, g) : 0.0;
        }
        return;
    }
    it -= m.D;
    if (it < m.D) {
        // row i of L^T L: (L^T L)(i,j) = sum over shared rows k (ascending) of L(k,i) L(k,j)
        int i = it;
        const PlaneGeom gi = pg[m.lt_plane[i]];
        double vi[9];
        int ri[9];
        for (int q = 0; q < 9; ++q) {
            ri[q] = m.lt_row[i * 9 + q];
            vi[q] = ri[q] >= 0 ? stencil_value(m.lt_k + (i * 9 + q) * 3, gi) : 0.0;
        }
        for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) {
            int j = m.ll_col[e];
            const PlaneGeom gj = pg[m.lt_plane[j]];
            double s = 0.0;
            int a = 0, b = 0;
            while (a < 9 && b < 9 && ri[a] >= 0 && m.lt_row[j * 9 + b] >= 0) {
                int rb = m.lt_row[j * 9 + b];
                if (ri[a] == rb) {
                    s += vi[a] * stencil_value(m.lt_k + (j * 9 + b) * 3, gj);
                    ++a; ++b;
                } else if (ri[a] < rb) {
                    ++a;
                } else {
                    ++b;
                }
            }
            llval[(size_t)th * m.ll_nnz + e] = s;
        }
        return;
    }
    // hyper-parameters (get_sigma)
    const double *tt = theta + (size_t)th * m.ndim_fault;
    double la2, lsar, lgnss;
    int n = m.nplane;
    if (m.layout == SMCGPU_LAYOUT_RECT) {
        la2 = tt[7];
        lsar = m.rect_hyper ? tt[8] : 0.0;
        lgnss = m.rect_hyper ? tt[9] : 0.0;
    } else if (m.layout == SMCGPU_LAYOUT_TRACE_FIXBEND) {
        la2 = tt[2 * n + 1]; lsar = tt[2 * n + 2]; lgnss = tt[2 * n + 3];
    } else {
        la2 = tt[3 * n]; lsar = tt[3 * n + 1]; lgnss = tt[3 * n + 2];
    }
    ThetaAux a;
    a.log_alpha2 = la2;
    a.log_sigma_sar2 = lsar;
    a.log_sigma_gnss2 = lgnss;
    a.alpha2 = exp(la2);
    a.sigma_sar2 = exp(lsar);
    a.sigma_gnss2 = exp(lgnss);
    a.lconst = m.nsar * lsar / 2.0 + 3.0 * m.ngnss * lgnss / 2.0;
    aux[th] = a;
}

cudaError_t launch_setup(const MeshDev &m, int n_theta, const double *theta_dev, const PlaneGeom *planes_dev,
                         double *lval, double *ltval, double *llval, ThetaAux *aux, cudaStream_t s) {
    long long n = (long long)n_theta * (m.nrow + 2 * m.D + 1);
    if (n <= 0) return cudaSuccess;
    setup_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, n_theta, theta_dev, planes_dev, lval, ltval, llval, aux);
    return cudaGetLastError();
}

}  // namespace smc
