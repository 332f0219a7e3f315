// Gram precompute of slip_calc_gsd_gsg (smc_slip.f90:1347-1443):
//   A = G^T Sigma^-1 G,  b = G^T Sigma^-1 d,  dsd = d^T Sigma^-1 d
// with Sigma^-1 = diag(1/(sigma_i^2 sigma2_gnss)) on GNSS rows and
// Sigma_SAR,p^-1 / sigma2_sar on each InSAR path.  The InSAR blocks are
// applied through their whitening factor W_p (W_p^T W_p = Sigma_SAR,p^-1,
// computed once from the data), so A and b come from the whitened rows.
#include "common.cuh"
#include "kernels.h"
#include "mesh.h"

namespace smc {

// Gw[th][col][row] = sum_k<=row W_p(row, k) G[th][col][st_p + k]
__global__ void whiten_kernel(MeshDev m, int n_theta, const double *__restrict__ gmat, double *__restrict__ gw) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long per = (long long)m.D * m.nsar;
    if (t >= (long long)n_theta * per) return;
    int th = (int)(t / per);
    int rem = (int)(t % per);
    int col = rem / m.nsar, row = rem % m.nsar;
    int p = 0;
    while (p + 1 < m.npath && m.nsar_index[p + 1] <= row) ++p;
    int st = m.nsar_index[p], n = m.nsar_index[p + 1] - st, i = row - st;
    const double *W = m.sar_inv + m.sar_off[p];
    const double *g = gmat + ((size_t)th * m.D + col) * m.nobs + st;
    double s = 0.0;
    for (int k = 0; k <= i; ++k) s += W[(size_t)k * n + i] * g[k];
    gw[((size_t)th * m.D + col) * m.nsar + row] = s;
}

__device__ __forceinline__ const double *gx_col(const MeshDev &m, const double *gmat, const double *gw, int th, int c,
                                                bool sar) {
    return sar ? gw + ((size_t)th * m.D + c) * m.nsar : gmat + ((size_t)th * m.D + c) * m.nobs;
}

// A(i,j), j <= i, mirrored; b(i) and dsd in the last items of each theta
__global__ void gram_kernel(MeshDev m, int n_theta, const double *__restrict__ gmat, const double *__restrict__ gw,
                            const double *__restrict__ roww, const double *__restrict__ dx,
                            const ThetaAux *__restrict__ aux, double dsd_sar, double dsd_gnss,
                            double *__restrict__ A, double *__restrict__ b, double *__restrict__ dsd) {
    const int D = m.D;
    const long long npair = (long long)D * (D + 1) / 2;
    const long long per = npair + D + 1;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_theta * per) return;
    int th = (int)(t / per);
    long long it = t % per;
    const ThetaAux ax = aux[th];
    const double ssar = 1.0 / ax.sigma_sar2, sgnss = 1.0 / ax.sigma_gnss2;
    if (it < npair) {
        // unrank the lower-triangle pair (i, j), j <= i
        int i = (int)((sqrt(8.0 * (double)it + 1.0) - 1.0) / 2.0);
        while ((long long)i * (i + 1) / 2 > it) --i;
        while ((long long)(i + 1) * (i + 2) / 2 <= it) ++i;
        int j = (int)(it - (long long)i * (i + 1) / 2);
        double s_sar = 0.0, s_gn = 0.0;
        if (m.nsar > 0) {
            const double *gi = gx_col(m, gmat, gw, th, i, true), *gj = gx_col(m, gmat, gw, th, j, true);
            for (int r = 0; r < m.nsar; ++r) s_sar += gi[r] * gj[r];
        }
        const double *gi = gmat + ((size_t)th * D + i) * m.nobs, *gj = gmat + ((size_t)th * D + j) * m.nobs;
        for (int r = m.nsar; r < m.nobs; ++r) s_gn += roww[r] * gi[r] * gj[r];
        double v = s_sar * ssar + s_gn * sgnss;
        double *Ath = A + (size_t)th * D * D;
        Ath[(size_t)j * D + i] = v;
        Ath[(size_t)i * D + j] = v;
        return;
    }
    it -= npair;
    if (it < D) {
        int i = (int)it;
        double s_sar = 0.0, s_gn = 0.0;
        if (m.nsar > 0) {
            const double *gi = gx_col(m, gmat, gw, th, i, true);
            for (int r = 0; r < m.nsar; ++r) s_sar += gi[r] * dx[r];
        }
        const double *gi = gmat + ((size_t)th * D + i) * m.nobs;
        for (int r = m.nsar; r < m.nobs; ++r) s_gn += roww[r] * gi[r] * dx[r];
        b[(size_t)th * D + i] = s_sar * ssar + s_gn * sgnss;
        return;
    }
    dsd[th] = dsd_sar * ssar + dsd_gnss * sgnss;
}

cudaError_t launch_gram(const MeshDev &m, int n_theta, const double *gmat, const double *roww, const double *dx,
                             const ThetaAux *aux, double dsd_sar, double dsd_gnss, double *A, double *b, double *dsd,
                             double *gw, cudaStream_t s) {
    if (n_theta <= 0) return cudaSuccess;
    if (m.nsar > 0) {
        long long n = (long long)n_theta * m.D * m.nsar;
        whiten_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, n_theta, gmat, gw);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    long long per = (long long)m.D * (m.D + 1) / 2 + m.D + 1;
    long long n = (long long)n_theta * per;
    gram_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, n_theta, gmat, gw, roww, dx, aux, dsd_sar, dsd_gnss, A,
                                                             b, dsd);
    return cudaGetLastError();
}

}  // namespace smc
