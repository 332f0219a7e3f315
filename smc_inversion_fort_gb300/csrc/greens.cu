// Batched Green's-function build: Okada (1992) point sources DC3D0 over
// (theta x plane x patch x Gauss point x station), the GB300 restatement of
// calc_greens_func / calc_responce_dist / calc_responce / call_dc3d0
// (gfunc.f90:65-348) and DC3D0 (DC3Dfortran.f90:2-607).
//
// One thread owns one (theta, station) pair and sweeps the sources of every
// plane, so each DC3D0 evaluation is done once for both slip directions and
// scattered to its basis columns (the reference re-evaluates every
// (patch, Gauss point, station) for every touching node and direction).
// Geometry is expressed in the fault frame of each plane:
//   x = x_st - xi,  y = y_st - eta*cos(dip),  depth = -(zf + eta*sin(dip)),
// with (x_st, y_st) the station rotated into the strike frame about the
// plane centre (algebraically identical to gfunc.f90:80-81, 175-179).
// With z = 0 the real-source and image UA0 terms of DC3D0 cancel and UC0 is
// multiplied by z, so the displacement is UB0's (DC3Dfortran.f90:273-442).
#include "common.cuh"
#include "kernels.h"
#include "mesh.h"

namespace smc {

__device__ void plane_geometry(const MeshDev &m, const double *th, int ip, PlaneGeom &g) {
    const double pi = 3.141592653589793;  // 4*atan(1), 2*asin(1)
    double strike, dip, xf, yf, zf, lxi, leta;
    if (m.layout == SMCGPU_LAYOUT_RECT) {
        dip = th[6];
        strike = th[5];
        double dip_rad = dip * pi / 180.0;
        xf = th[0];
        yf = th[1];
        zf = -(th[2] + th[4] / 2.0 * sin(dip_rad));
        lxi = th[3];
        leta = th[4];
    } else {
        // get_geometry (init.f90:121-173) and fault centre (gfunc.f90:290-296)
        int n = m.nplane, p1 = ip + 1;
        double ymin = th[0], ymax = th[1], xl, yl, xr, yr;
        if (m.layout == SMCGPU_LAYOUT_TRACE_FIXBEND) {
            if (p1 == 1) { xl = m.xmin; yl = ymin; } else { xl = m.xbend[p1 - 2]; yl = th[p1]; }
            if (p1 == n) { xr = m.xmax; yr = ymax; } else { xr = m.xbend[p1 - 1]; yr = th[p1 + 1]; }
            dip = th[n + p1];
        } else {
            if (p1 == 1) { xl = m.xmin; yl = ymin; } else { xl = th[2 * p1 - 2]; yl = th[2 * p1 - 1]; }
            if (p1 == n) { xr = m.xmax; yr = ymax; } else { xr = th[2 * p1]; yr = th[2 * p1 + 1]; }
            dip = th[2 * n + p1 - 1];
        }
        double dip_rad = dip * pi / 180.0;
        lxi = sqrt((xr - xl) * (xr - xl) + (yr - yl) * (yr - yl));
        leta = -m.zmin / sin(dip_rad);
        double strike_rad = atan2(xr - xl, yr - yl);
        strike = strike_rad / pi * 180.0;
        xf = (xl + xr) / 2.0 - (m.zmin * cos(strike_rad)) / (2.0 * tan(dip_rad));
        yf = (yl + yr) / 2.0 + (m.zmin * sin(strike_rad)) / (2.0 * tan(dip_rad));
        zf = m.zmin / 2.0;
    }
    g.xf = xf; g.yf = yf; g.zf = zf;
    g.strike = strike; g.dip = dip; g.lxi = lxi; g.leta = leta;
    double sr = strike / 180.0 * pi, dr = dip / 180.0 * pi;
    g.sin_s = sin(sr); g.cos_s = cos(sr);
    g.cos_dip = cos(dr); g.sin_dip = sin(dr);
    // DCCON0
    const double P18 = 6.283185307179586 / 360.0;
    double sd = sin(dip * P18), cd = cos(dip * P18);
    if (fabs(cd) < 1.0e-6) { cd = 0.0; if (sd > 0.0) sd = 1.0; if (sd < 0.0) sd = -1.0; }
    g.sd = sd; g.cd = cd;
    g.dxi = lxi / m.nxi[ip];
    g.deta = leta / m.neta[ip];
}

__global__ void planes_kernel(MeshDev m, int n_theta, const double *__restrict__ theta, PlaneGeom *__restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_theta * m.nplane) return;
    int th = t / m.nplane, ip = t % m.nplane;
    PlaneGeom g;
    plane_geometry(m, theta + (size_t)th * m.ndim_fault, ip, g);
    out[t] = g;
}

// UB0 displacement terms (DC3Dfortran.f90:314-400, components 1-3) for unit
// strike and dip potency, z = 0 so C = D.  Not yet divided by 2*pi.
template <typename T>
__device__ __forceinline__ void ub0_disp(T X, T Y, T D, T SD, T CD, T aSD, T aSC, T us[3], T ud[3]);

template <>
__device__ __forceinline__ void ub0_disp<double>(double X, double Y, double D, double SD, double CD, double aSD,
                                                 double aSC, double us[3], double ud[3]) {
    // one reciprocal square root instead of a square root and a division
    // (about 1 ulp; the FP64 pipe is this kernel's bound)
    const double R2 = X * X + Y * Y + D * D;
    const double iR = rsqrt(R2);
    const double R = R2 * iR;
    double P = Y * CD + D * SD, Q = Y * SD - D * CD;
    double RD = R + D, iRD = 1.0 / RD;
    double iR2 = iR * iR, iR3 = iR2 * iR, iR5 = iR3 * iR2;
    double QR = 3.0 * Q * iR5;
    double D12 = iR * iRD * iRD;
    double D32 = D12 * (2.0 * R + D) * iR2;
    double D33 = D12 * (3.0 * R + D) * iR2 * iRD;
    double X2 = X * X, Y2 = Y * Y, XY = X * Y;
    double FI1 = Y * (D12 - X2 * D33);
    double FI2 = X * (D12 - Y2 * D33);
    double FI3 = X * iR3 - FI2;
    double FI4 = -XY * D32;
    double FI5 = iR * iRD - X2 * D32;
    // aSD = alp3 SD, aSC = alp3 SD CD: per-plane constants
    us[0] = -X2 * QR - aSD * FI1;
    us[1] = -XY * QR - aSD * FI2;
    us[2] = -D * X * QR - aSD * FI4;
    const double PQR = P * QR;
    ud[0] = -X * PQR + aSC * FI3;
    ud[1] = -Y * PQR + aSC * FI1;
    ud[2] = -D * PQR + aSC * FI5;
}

// FP32: reciprocal square root and the cancellation-free form of
// FI3 = X/R^3 - FI2 = X*(D*(2R+D)/(R^3 RD^2) + Y^2 D33).
template <>
__device__ __forceinline__ void ub0_disp<float>(float X, float Y, float D, float SD, float CD, float aSD,
                                                float aSC, float us[3], float ud[3]) {
    float R2 = fmaf(X, X, fmaf(Y, Y, D * D));
    float iR = rsqrtf(R2);
    float R = R2 * iR;
    float P = fmaf(Y, CD, D * SD), Q = fmaf(Y, SD, -D * CD);
    float RD = R + D, iRD = __frcp_rn(RD);
    float iR2 = iR * iR, iR3 = iR2 * iR, iR5 = iR3 * iR2;
    float QR = 3.0f * Q * iR5;
    float D12 = iR * iRD * iRD;
    float tR = 2.0f * R + D;
    float D32 = D12 * tR * iR2;
    float D33 = D12 * (3.0f * R + D) * iR2 * iRD;
    float X2 = X * X, Y2 = Y * Y, XY = X * Y;
    float FI1 = Y * fmaf(-X2, D33, D12);
    float FI2 = X * fmaf(-Y2, D33, D12);
    float FI3 = X * fmaf(Y2, D33, D * tR * iR3 * iRD * iRD);
    float FI4 = -XY * D32;
    float FI5 = fmaf(-X2, D32, iR * iRD);
    us[0] = fmaf(-X2, QR, -aSD * FI1);
    us[1] = fmaf(-XY, QR, -aSD * FI2);
    us[2] = fmaf(-D * X, QR, -aSD * FI4);
    ud[0] = fmaf(-X * P, QR, aSC * FI3);
    ud[1] = fmaf(-Y * P, QR, aSC * FI1);
    ud[2] = fmaf(-D * P, QR, aSC * FI5);
}

// DC3D0 displacement at one receiver for unit strike / dip potency, with the
// reference's guards: depth < 0 returns zero (DC3Dfortran.f90:67-70),
// |x|,|y|,|d| < 1e-6 are snapped to zero (:71-73), R == 0 returns zero (:82-85).
template <typename T>
__device__ __forceinline__ bool dc3d0_disp(T x, T y, T depth, T SD, T CD, T aSD, T aSC, T us[3], T ud[3]) {
    if (depth < T(0)) return false;
    const T EPS = T(1.0e-6);
    if (fabs(x) < EPS) x = T(0);
    if (fabs(y) < EPS) y = T(0);
    if (fabs(depth) < EPS) depth = T(0);
    if (x == T(0) && y == T(0) && depth == T(0)) return false;
    ub0_disp<T>(x, y, depth, SD, CD, aSD, aSC, us, ud);
    return true;
}
// FP64: the same guards as integer tests on the bit patterns (the comparisons
// would otherwise occupy the FP64 pipe): |v| < 1e-6 is |bits| < bits(1e-6)
// for finite and NaN v alike, and depth < 0 is a set sign bit on a nonzero,
// non-NaN value.
template <>
__device__ __forceinline__ bool dc3d0_disp<double>(double x, double y, double depth, double SD, double CD,
                                                   double aSD, double aSC, double us[3], double ud[3]) {
    const unsigned long long MAG = 0x7FFFFFFFFFFFFFFFull, INF = 0x7FF0000000000000ull;
    const unsigned long long EPSB = 0x3EB0C6F7A0B5ED8Dull;   // 1.0e-6
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
    const unsigned long long by = (unsigned long long)__double_as_longlong(y);
    const unsigned long long bd = (unsigned long long)__double_as_longlong(depth);
    if ((bd >> 63) && (bd & MAG) != 0 && (bd & MAG) <= INF) return false;
    const bool zx = (bx & MAG) < EPSB, zy = (by & MAG) < EPSB, zd = (bd & MAG) < EPSB;
    if (zx && zy && zd) return false;
    ub0_disp<double>(zx ? 0.0 : x, zy ? 0.0 : y, zd ? 0.0 : depth, SD, CD, aSD, aSC, us, ud);
    return true;
}

template <typename T, typename OutT>
__device__ __forceinline__ void write_column(const MeshDev &m, OutT *__restrict__ g, int col, int row0, int nrow,
                                             const T acc[3], T sin_s, T cos_s, T scale) {
    // inverse rotation + cm scaling (gfunc.f90:93-99), then the LOS dot
    // product of calc_greens_func (gfunc.f90:320-326)
    T ux = scale * (sin_s * acc[0] - cos_s * acc[1]);
    T uy = scale * (cos_s * acc[0] + sin_s * acc[1]);
    T uz = scale * acc[2];
    OutT *gc = g + (size_t)col * m.nobs;
    for (int r = 0; r < nrow; ++r) {
        const double *e = m.obs_e + 3 * (row0 + r);
        T v = ux * (T)e[0] + uy * (T)e[1] + uz * (T)e[2];
        gc[row0 + r] = (OutT)v;
    }
}

template <typename T, typename OutT, int BASIS>
__global__ void __launch_bounds__(128) greens_kernel(MeshDev m, int n_theta, const PlaneGeom *__restrict__ planes,
                                                     OutT *__restrict__ gmat) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_theta * m.nstation) return;
    int th = (int)(t / m.nstation), st = (int)(t % m.nstation);
    double xo = m.st_x[st], yo = m.st_y[st];
    int row0 = m.st_row[st], nrow = m.st_nrow[st];
    OutT *g = gmat + (size_t)th * m.D * m.nobs;
    const T alp3 = (T)((1.0 - m.alpha) / m.alpha);
    const T scale = (T)(100.0 / 6.283185307179586);
    int nq = m.nquad;
    T qx[MAXQ], qw[MAXQ];
    for (int a = 0; a < nq; ++a) { qx[a] = (T)((1.0 + m.gq_x[a]) * 0.5); qw[a] = (T)m.gq_w[a]; }
    // rolling node accumulators of the nodal basis: pending contributions of
    // the node row above the current patch row, per node column
    T pend[BASIS == 0 ? 33 * 6 : 1];
    for (int ip = 0; ip < m.nplane; ++ip) {
        const PlaneGeom pg = planes[(size_t)th * m.nplane + ip];
        double dx0 = xo - pg.xf, dy0 = yo - pg.yf;
        T xs = (T)(pg.sin_s * dx0 + pg.cos_s * dy0);
        T ys = (T)(-pg.cos_s * dx0 + pg.sin_s * dy0);
        T cdip = (T)pg.cos_dip, sdip = (T)pg.sin_dip, SD = (T)pg.sd, CD = (T)pg.cd;
        T zf = (T)pg.zf, sin_s = (T)pg.sin_s, cos_s = (T)pg.cos_s;
        int nxi = m.nxi[ip], neta = m.neta[ip];
        T dxi = (T)pg.dxi, deta = (T)pg.deta;
        T lxi2 = (T)(pg.lxi / 2.0), leta2 = (T)(pg.leta / 2.0);
        T area = dxi * deta;
        const T aSD = alp3 * SD, aSC = alp3 * SD * CD;
        T wa[MAXQ];   // area * w_a / 4 (the quadrature weight w_b completes it)
        for (int a = 0; a < nq; ++a) wa[a] = area * qw[a] * T(0.25);
        if (BASIS == 0)
            for (int q = 0; q < (nxi + 1) * 6; ++q) pend[q] = T(0);
        for (int j = 0; j < neta; ++j) {
            T eta0 = (T)j * deta - leta2;
            // receiver offsets along dip for this patch row's Gauss points
            T yb[MAXQ], db[MAXQ];
            for (int b = 0; b < nq; ++b) {
                const T eta = eta0 + qx[b] * deta;
                yb[b] = ys - eta * cdip;
                db[b] = -(zf + eta * sdip);
            }
            T carry_b[6], carry_t[6];
            for (int q = 0; q < 6; ++q) { carry_b[q] = T(0); carry_t[q] = T(0); }
            for (int i = 0; i < nxi; ++i) {
                T xi0 = (T)i * dxi - lxi2;
                // corner accumulators: 0 BL (i,j), 1 BR (i+1,j), 2 TR (i+1,j+1), 3 TL (i,j+1)
                T acc[BASIS == 0 ? 4 : 1][6];
                for (int c = 0; c < (BASIS == 0 ? 4 : 1); ++c)
                    for (int q = 0; q < 6; ++q) acc[c][q] = T(0);
                for (int a = 0; a < nq; ++a) {
                    T xi = xi0 + qx[a] * dxi;
                    T x = xs - xi;
                    for (int b = 0; b < nq; ++b) {
                        T us[3], ud[3];
                        if (!dc3d0_disp<T>(x, yb[b], db[b], SD, CD, aSD, aSC, us, ud)) continue;
                        T w = wa[a] * qw[b];
                        if (BASIS == 0) {
                            T r1 = (T)m.gq_x[a], r2 = (T)m.gq_x[b];
                            T nv[4] = {(T(1) - r1) * (T(1) - r2) * T(0.25), (T(1) + r1) * (T(1) - r2) * T(0.25),
                                       (T(1) + r1) * (T(1) + r2) * T(0.25), (T(1) - r1) * (T(1) + r2) * T(0.25)};
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                T wc = w * nv[c];
#pragma unroll
                                for (int q = 0; q < 3; ++q) {
                                    acc[c][q] += wc * us[q];
                                    acc[c][3 + q] += wc * ud[q];
                                }
                            }
                        } else {
#pragma unroll
                            for (int q = 0; q < 3; ++q) {
                                acc[0][q] += w * us[q];
                                acc[0][3 + q] += w * ud[q];
                            }
                        }
                    }
                }
                if (BASIS == 1) {
                    int col = 2 * (m.patch_off[ip] + i + nxi * j);
                    write_column<T, OutT>(m, g, col, row0, nrow, acc[0], sin_s, cos_s, -scale);
                    write_column<T, OutT>(m, g, col + 1, row0, nrow, acc[0] + 3, sin_s, cos_s, scale);
                } else {
                    // node (i, j) is complete: pending from the row below,
                    // bottom-right of patch i-1 and bottom-left of patch i
                    T node[6];
                    for (int q = 0; q < 6; ++q) node[q] = pend[i * 6 + q] + carry_b[q] + acc[0][q];
                    int dof = m.dof_of_node[m.node_off[ip] + i + (nxi + 1) * j];
                    if (dof >= 0) {
                        write_column<T, OutT>(m, g, 2 * dof, row0, nrow, node, sin_s, cos_s, -scale);
                        write_column<T, OutT>(m, g, 2 * dof + 1, row0, nrow, node + 3, sin_s, cos_s, scale);
                    }
                    for (int q = 0; q < 6; ++q) {
                        pend[i * 6 + q] = carry_t[q] + acc[3][q];
                        carry_b[q] = acc[1][q];
                        carry_t[q] = acc[2][q];
                    }
                }
            }
            if (BASIS == 0) {
                T node[6];
                for (int q = 0; q < 6; ++q) node[q] = pend[nxi * 6 + q] + carry_b[q];
                int dof = m.dof_of_node[m.node_off[ip] + nxi + (nxi + 1) * j];
                if (dof >= 0) {
                    write_column<T, OutT>(m, g, 2 * dof, row0, nrow, node, sin_s, cos_s, -scale);
                    write_column<T, OutT>(m, g, 2 * dof + 1, row0, nrow, node + 3, sin_s, cos_s, scale);
                }
                for (int q = 0; q < 6; ++q) pend[nxi * 6 + q] = carry_t[q];
            }
        }
        if (BASIS == 0) {  // top node row
            for (int i = 0; i <= nxi; ++i) {
                int dof = m.dof_of_node[m.node_off[ip] + i + (nxi + 1) * neta];
                if (dof < 0) continue;
                write_column<T, OutT>(m, g, 2 * dof, row0, nrow, pend + i * 6, sin_s, cos_s, -scale);
                write_column<T, OutT>(m, g, 2 * dof + 1, row0, nrow, pend + i * 6 + 3, sin_s, cos_s, scale);
            }
        }
    }
}

cudaError_t launch_planes(const MeshDev &m, int n_theta, const double *theta_dev, PlaneGeom *planes_dev,
                          cudaStream_t s) {
    int n = n_theta * m.nplane;
    if (n <= 0) return cudaSuccess;
    planes_kernel<<<(n + 127) / 128, 128, 0, s>>>(m, n_theta, theta_dev, planes_dev);
    return cudaGetLastError();
}

cudaError_t launch_greens(const MeshDev &m, int n_theta, const PlaneGeom *planes_dev, int precision, void *gmat_dev,
                          cudaStream_t s) {
    long long n = (long long)n_theta * m.nstation;
    if (n <= 0) return cudaSuccess;
    unsigned blocks = (unsigned)((n + 127) / 128);
    if (precision == SMCGPU_PREC_FP32) {
        if (m.basis == SMCGPU_BASIS_NODAL)
            greens_kernel<float, float, 0><<<blocks, 128, 0, s>>>(m, n_theta, planes_dev, (float *)gmat_dev);
        else
            greens_kernel<float, float, 1><<<blocks, 128, 0, s>>>(m, n_theta, planes_dev, (float *)gmat_dev);
    } else {
        if (m.basis == SMCGPU_BASIS_NODAL)
            greens_kernel<double, double, 0><<<blocks, 128, 0, s>>>(m, n_theta, planes_dev, (double *)gmat_dev);
        else
            greens_kernel<double, double, 1><<<blocks, 128, 0, s>>>(m, n_theta, planes_dev, (double *)gmat_dev);
    }
    return cudaGetLastError();
}

}  // namespace smc
