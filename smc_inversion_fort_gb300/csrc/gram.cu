// Gram precompute of slip_calc_gsd_gsg (smc_slip.f90:1347-1443):
//   A = G^T Sigma^-1 G,  b = G^T Sigma^-1 d,  dsd = d^T Sigma^-1 d
// with Sigma^-1 = diag(1/(sigma_i^2 sigma2_gnss)) on GNSS rows and
// Sigma_SAR,p^-1 / sigma2_sar on each InSAR path.  The InSAR blocks are
// applied through their whitening factor W_p (W_p^T W_p = Sigma_SAR,p^-1,
// computed once from the data), so A and b come from the whitened rows.
#include "common.cuh"
#include "kernels.h"
#include "mesh.h"

#include <algorithm>

namespace smc {

// Both products are FP64 and bound by the FP64 pipe.  They run as 64 x 64
// output tiles (16 x 16 threads, 4 x 4 outputs each, 16-row K chunks staged in
// shared memory); every output still accumulates its terms one at a time in
// increasing row order, so the tiles change no bit of the result.
constexpr int GT = 64, GK = 16;

// Gw[th][col][st_p + i] = sum_{k <= i} W_p(i, k) G[th][col][st_p + k] for every
// path p: per path one product W_p (n x n, lower triangle) times the n x (n_theta D)
// block of G rows st_p .. st_p + n - 1 (columns j = th D + col, stride nobs).
__global__ void __launch_bounds__(256) whiten_kernel(MeshDev m, int ncols, const double *__restrict__ gmat,
                                                     double *__restrict__ gw) {
    __shared__ double Ws[GK][GT], Xs[GK][GT + 1];
    const int p = blockIdx.z;
    const int st = m.nsar_index[p], n = m.nsar_index[p + 1] - st;
    const int i0 = blockIdx.y * GT, j0 = blockIdx.x * GT;
    if (i0 >= n) return;
    const double *W = m.sar_inv + m.sar_off[p];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
    const int kend = min(n, i0 + GT);   // W(i, k) = 0 for k > i
    for (int k0 = 0; k0 < kend; k0 += GK) {
        for (int q = threadIdx.x; q < GK * GT; q += 256) {
            const int kk = q / GT, ii = q % GT, k = k0 + kk, i = i0 + ii;
            Ws[kk][ii] = (k < n && i < n && k <= i) ? W[(size_t)k * n + i] : 0.0;
            const int jj = q / GK, kx = q % GK, j = j0 + jj;
            Xs[kx][jj] = (k0 + kx < n && j < ncols) ? gmat[(size_t)j * m.nobs + st + k0 + kx] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            double wv[4], xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) wv[u] = Ws[kk][ty + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) xv[v] = Xs[kk][tx + 16 * v];
            // a zero W entry (k > i) adds an exact zero to the sum
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(wv[u], xv[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
            if (i < n && j < ncols) gw[(size_t)j * m.nsar + st + i] = acc[u][v];
        }
}

// A(i, j) for j <= i (mirrored) over the lower-triangle 64 x 64 tiles of one
// geometry: sum_r Gw(r, i) Gw(r, j) / sigma2_sar + sum_r roww(r) G(r, i) G(r, j) / sigma2_gnss
__global__ void __launch_bounds__(256) gram_kernel(MeshDev m, const double *__restrict__ gmat,
                                                   const double *__restrict__ gw, const double *__restrict__ roww,
                                                   const ThetaAux *__restrict__ aux, double *__restrict__ A, int th0) {
    __shared__ double Is[GK][GT + 1], Js[GK][GT + 1], Rw[GK];
    const int D = m.D, th = th0 + (int)blockIdx.y;
    // unrank the tile pair (bi, bj), bj <= bi
    int bi = 0, t = blockIdx.x;
    while (t > bi) { t -= bi + 1; ++bi; }
    const int bj = t, i0 = bi * GT, j0 = bj * GT;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double ssum[4][4], gsum[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) ssum[u][v] = gsum[u][v] = 0.0;
    // InSAR rows from the whitened columns, then GNSS rows weighted by roww
    for (int part = 0; part < 2; ++part) {
        const bool sar = part == 0;
        const int r0 = sar ? 0 : m.nsar, r1 = sar ? m.nsar : m.nobs, ld = sar ? m.nsar : m.nobs;
        const double *X = sar ? gw + (size_t)th * D * m.nsar : gmat + (size_t)th * D * m.nobs;
        for (int k0 = r0; k0 < r1; k0 += GK) {
            for (int q = threadIdx.x; q < GK * GT; q += 256) {
                const int cc = q / GK, kx = q % GK, r = k0 + kx;
                Is[kx][cc] = (r < r1 && i0 + cc < D) ? X[(size_t)(i0 + cc) * ld + r] : 0.0;
                Js[kx][cc] = (r < r1 && j0 + cc < D) ? X[(size_t)(j0 + cc) * ld + r] : 0.0;
            }
            if (!sar && threadIdx.x < GK) Rw[threadIdx.x] = k0 + threadIdx.x < r1 ? roww[k0 + threadIdx.x] : 0.0;
            __syncthreads();
            const int kn = min(GK, r1 - k0);
            if (sar) {
                for (int kk = 0; kk < kn; ++kk) {
                    double iv[4], jv[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) iv[u] = Is[kk][ty + 16 * u];
#pragma unroll
                    for (int v = 0; v < 4; ++v) jv[v] = Js[kk][tx + 16 * v];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v) ssum[u][v] = fma(iv[u], jv[v], ssum[u][v]);
                }
            } else {
                for (int kk = 0; kk < kn; ++kk) {
                    const double rw = Rw[kk];
                    double iv[4], jv[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) iv[u] = rw * Is[kk][ty + 16 * u];   // roww(r) G(r, i), i >= j
#pragma unroll
                    for (int v = 0; v < 4; ++v) jv[v] = Js[kk][tx + 16 * v];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v) gsum[u][v] = fma(iv[u], jv[v], gsum[u][v]);
                }
            }
            __syncthreads();
        }
    }
    const ThetaAux ax = aux[th];
    const double ssar = 1.0 / ax.sigma_sar2, sgnss = 1.0 / ax.sigma_gnss2;
    double *Ath = A + (size_t)th * D * D;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
            if (i < D && j <= i) {
                const double s_sar = ssum[u][v], s_gn = gsum[u][v];
                const double val = s_sar * ssar + s_gn * sgnss;
                Ath[(size_t)j * D + i] = val;
                Ath[(size_t)i * D + j] = val;
            }
        }
}

// b(i) = G^T Sigma^-1 d (whitened InSAR rows, weighted GNSS rows) and dsd
__global__ void gsd_kernel(MeshDev m, int n_theta, const double *__restrict__ gmat, const double *__restrict__ gw,
                           const double *__restrict__ roww, const double *__restrict__ dx,
                           const ThetaAux *__restrict__ aux, double dsd_sar, double dsd_gnss, double *__restrict__ b,
                           double *__restrict__ dsd) {
    const int D = m.D;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_theta * (D + 1)) return;
    const int th = (int)(t / (D + 1)), i = (int)(t % (D + 1));
    const ThetaAux ax = aux[th];
    const double ssar = 1.0 / ax.sigma_sar2, sgnss = 1.0 / ax.sigma_gnss2;
    if (i == D) { dsd[th] = dsd_sar * ssar + dsd_gnss * sgnss; return; }
    double s_sar = 0.0, s_gn = 0.0;
    if (m.nsar > 0) {
        const double *gi = gw + ((size_t)th * D + i) * m.nsar;
        for (int r = 0; r < m.nsar; ++r) s_sar += gi[r] * dx[r];
    }
    const double *gi = gmat + ((size_t)th * D + i) * m.nobs;
    for (int r = m.nsar; r < m.nobs; ++r) s_gn += roww[r] * gi[r] * dx[r];
    b[(size_t)th * D + i] = s_sar * ssar + s_gn * sgnss;
}

cudaError_t launch_gram(const MeshDev &m, int n_theta, const double *gmat, const double *roww, const double *dx,
                             const ThetaAux *aux, double dsd_sar, double dsd_gnss, double *A, double *b, double *dsd,
                             double *gw, cudaStream_t s) {
    if (n_theta <= 0) return cudaSuccess;
    const int ncols = n_theta * m.D;
    if (m.nsar > 0) {
        const dim3 grid((unsigned)((ncols + GT - 1) / GT), (unsigned)((m.nsar + GT - 1) / GT), (unsigned)m.npath);
        whiten_kernel<<<grid, 256, 0, s>>>(m, ncols, gmat, gw);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int nb = (m.D + GT - 1) / GT;
    for (int th0 = 0; th0 < n_theta; th0 += 65535) {   // grid y limit
        const int nth = std::min(65535, n_theta - th0);
        gram_kernel<<<dim3((unsigned)(nb * (nb + 1) / 2), (unsigned)nth), 256, 0, s>>>(m, gmat, gw, roww, aux, A, th0);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const long long n = (long long)n_theta * (m.D + 1);
    gsd_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, n_theta, gmat, gw, roww, dx, aux, dsd_sar, dsd_gnss, b,
                                                           dsd);
    return cudaGetLastError();
}

}  // namespace smc
