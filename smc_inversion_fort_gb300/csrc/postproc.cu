// Post-processing of sampled geometries (main.f90:553-830):
//  * calc_slip_map: the mean inner-SMC slip of each geometry (the mean over
//    the final inner population, main.f90:623-634);
//  * point_cloud: every patch split into nr x nr sub-points, each placed in
//    global coordinates with its bilinearly interpolated slip
//    (main.f90:711-781).
#include "common.cuh"
#include "kernels.h"

namespace smc {

namespace {

// mean over the N particles of each geometry, per dimension, in the
// reference's order (sum over particles, then one division)
__global__ void mean_particles_kernel(int n, int N, int D, const double *__restrict__ parts, double *__restrict__ out) {
    const int th = blockIdx.x;
    if (th >= n) return;
    const double *p = parts + (size_t)th * N * D;
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < N; ++k) s = s + p[(size_t)k * D + d];
        out[(size_t)th * D + d] = s / N;
    }
}

// one thread per (geometry, patch, sub-point); points[th][patch][ir1][ir2][6]
__global__ void point_cloud_kernel(MeshDev m, int n, const PlaneGeom *__restrict__ planes,
                                   const double *__restrict__ slip, int slip_stride, int nr,
                                   double *__restrict__ points) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)m.npatch * nr * nr;
    if (tid >= per * n) return;
    const int th = (int)(tid / per);
    const int rem = (int)(tid % per);
    const int patch = rem / (nr * nr), ir1 = (rem / nr) % nr, ir2 = rem % nr;
    int ip = 0;
    while (ip + 1 < m.nplane && patch >= m.patch_off[ip + 1]) ++ip;
    const PlaneGeom g = planes[(size_t)th * m.nplane + ip];
    const int nxi = m.nxi[ip], neta = m.neta[ip];
    const int lp = patch - m.patch_off[ip];
    const int i = lp % nxi, j = lp / nxi;   // zero-based patch position in the plane
    const double dxi = g.lxi / nxi, deta = g.leta / neta;
    // corner nodes n1..n4 (init.f90:268-276) and their (xi, eta)
    const double x1 = i * dxi - g.lxi / 2.0, x2 = (i + 1) * dxi - g.lxi / 2.0;
    const double e1 = j * deta - g.leta / 2.0, e2 = (j + 1) * deta - g.leta / 2.0;
    const double xin[4] = {x1, x2, x2, x1}, etan[4] = {e1, e1, e2, e2};
    double uxn[4], uen[4];
    const double *sl = slip + (size_t)th * slip_stride;
    if (m.basis == SMCGPU_BASIS_NODAL) {
        const int n1 = m.node_off[ip] + i + (nxi + 1) * j;
        const int nodes[4] = {n1, n1 + 1, n1 + 1 + nxi + 1, n1 + nxi + 1};
        for (int k = 0; k < 4; ++k) {
            uxn[k] = sl[2 * nodes[k]];
            uen[k] = sl[2 * nodes[k] + 1];
        }
    } else {
        for (int k = 0; k < 4; ++k) {
            uxn[k] = sl[2 * patch];
            uen[k] = sl[2 * patch + 1];
        }
    }
    // sub-point centres and bilinear shape functions (main.f90:692-697, 730-743)
    const double r1 = -1.0 + 1.0 / (double)nr + ir1 * 2.0 / (double)nr;
    const double r2 = -1.0 + 1.0 / (double)nr + ir2 * 2.0 / (double)nr;
    const double nv[4] = {(1.0 - r1) * (1.0 - r2) / 4.0, (1.0 + r1) * (1.0 - r2) / 4.0,
                          (1.0 + r1) * (1.0 + r2) / 4.0, (1.0 - r1) * (1.0 + r2) / 4.0};
    double xi = 0.0, eta = 0.0, uxi = 0.0, ueta = 0.0;
    for (int k = 0; k < 4; ++k) {
        xi = xi + nv[k] * xin[k];
        eta = eta + nv[k] * etan[k];
        uxi = uxi + nv[k] * uxn[k];
        ueta = ueta + nv[k] * uen[k];
    }
    // global position of the point (main.f90:747-752)
    const double pi = 3.141592653589793;
    const double strike_rad = g.strike * pi / 180.0, dip_rad = g.dip * pi / 180.0;
    double *o = points + (size_t)tid * 6;
    o[0] = g.xf - eta * cos(dip_rad) * cos(strike_rad) + xi * sin(strike_rad);
    o[1] = g.yf + eta * cos(dip_rad) * sin(strike_rad) + xi * cos(strike_rad);
    o[2] = g.zf + eta * sin(dip_rad);
    o[3] = uxi;
    o[4] = ueta;
    o[5] = sqrt(uxi * uxi + ueta * ueta);
}

}  // namespace

cudaError_t launch_mean_particles(int n, int N, int D, const double *parts, double *out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    mean_particles_kernel<<<n, 128, 0, s>>>(n, N, D, parts, out);
    return cudaGetLastError();
}

cudaError_t launch_point_cloud(const MeshDev &m, int n, const PlaneGeom *planes, const double *slip, int slip_stride,
                               int nr, double *points, cudaStream_t s) {
    const long long total = (long long)n * m.npatch * nr * nr;
    if (total <= 0) return cudaSuccess;
    const int bs = 128;
    point_cloud_kernel<<<(unsigned)((total + bs - 1) / bs), bs, 0, s>>>(m, n, planes, slip, slip_stride, nr, points);
    return cudaGetLastError();
}

}  // namespace smc
