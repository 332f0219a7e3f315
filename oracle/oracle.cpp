// CPU oracle: plain C++ restatement of the reference's nested-SMC hot path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Each routine names the reference
// Fortran it restates (paths within KaiNakao/smc_inversion_fort).  Loop
// order, operation order, literal constants and the real(16) accumulators
// (here __float128) follow the reference; the Fortran intrinsic
// random_number is replaced by the counter-based Philox4x64-10 stream that
// the CUDA path also uses, so both can be driven by identical draws.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

// real(16): IEEE binary128.  AArch64 Linux's long double is binary128
// (software arithmetic in libgcc); on x86-64 GCC's __float128 + libquadmath.
#if defined(__aarch64__)
typedef long double quad;
static inline quad q_floor(quad x) { return floorl(x); }
static inline quad q_log(quad x) { return logl(x); }
#else
#include <quadmath.h>
typedef __float128 quad;
static inline quad q_floor(quad x) { return floorq(x); }
static inline quad q_log(quad x) { return logq(x); }
#endif

// ---------------------------------------------------------------------------
// Random stream (replaces random_number / random_number_correction,
// smc_slip.f90:8-24).  Philox4x64-10 (Salmon et al., SC'11), same bit
// stream as numpy.random.Philox with the counter pre-incremented.
// ---------------------------------------------------------------------------
static inline void mulhilo64(uint64_t a, uint64_t b, uint64_t *hi, uint64_t *lo) {
    unsigned __int128 p = (unsigned __int128)a * b;
    *hi = (uint64_t)(p >> 64);
    *lo = (uint64_t)p;
}

extern "C" void orc_philox4x64(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]) {
    uint64_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint64_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t hi0, lo0, hi1, lo1;
        mulhilo64(0xD2E7470EE14C6C93ull, c0, &hi0, &lo0);
        mulhilo64(0xCA5A826395121157ull, c2, &hi1, &lo1);
        uint64_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B97F4A7C15ull;
        k1 += 0xBB67AE8584CAA73Bull;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline uint64_t raw_draw(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                                uint64_t i, uint64_t j) {
    uint64_t ctr[4] = {((uint64_t)stage << 32) | purpose, i, j >> 2, 0};
    uint64_t key[2] = {seed, stream};
    uint64_t out[4];
    orc_philox4x64(ctr, key, out);
    return out[j & 3];
}

// random_number_correction: U[0,1) clipped below at 1e-5
extern "C" double orc_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                              uint64_t i, uint64_t j) {
    double x = (double)(raw_draw(seed, stream, purpose, stage, i, j) >> 11) * 0x1.0p-53;
    if (x < 1e-5) x = 1e-5;
    return x;
}

// slip_BoxMuller / fault_box_muller (smc_slip.f90:26-38, smc_fault.f90:357-370):
// only the sine branch p is used by every caller.
extern "C" double orc_normal(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                             uint64_t i, uint64_t d) {
    double pi = 2.0 * asin(1.0);
    double r = orc_uniform(seed, stream, purpose, stage, i, 2 * d);
    double s = orc_uniform(seed, stream, purpose, stage, i, 2 * d + 1);
    return sqrt(-2.0 * log(r)) * sin(2.0 * pi * s);
}

// random_number_correction_dd (smc_slip.f90:17-24): a real(16) uniform, here
// carried as an exact 106-bit double-double.
extern "C" void orc_quad_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                                 double *hi, double *lo) {
    uint64_t ctr[4] = {((uint64_t)stage << 32) | purpose, 0, 0, 0};
    uint64_t key[2] = {seed, stream};
    uint64_t out[4];
    orc_philox4x64(ctr, key, out);
    double h = (double)(out[0] >> 11) * 0x1.0p-53;
    double l = (double)(out[1] >> 11) * 0x1.0p-106;
    if ((quad)h + (quad)l < (quad)1e-5) { h = 1e-5; l = 0.0; }
    *hi = h; *lo = l;
}

enum {
    RNG_GIBBS = 1, RNG_TUNE_DTAU = 2, RNG_TUNE_MOM = 3, RNG_TUNE_MH = 4, RNG_TUNE_RES = 5,
    RNG_SMP_MOM = 6, RNG_SMP_MH = 7, RNG_RESAMPLE = 8,
    RNG_OUT_INIT = 16, RNG_OUT_RES = 17, RNG_OUT_PROP = 18, RNG_OUT_MH = 19, RNG_OUT_QINIT = 20
};
static const uint64_t OUTER_STREAM = ~0ull;
static inline uint64_t eval_stream(uint32_t iter, uint32_t kind, uint64_t slot) {
    return ((uint64_t)iter << 40) | ((uint64_t)kind << 39) | slot;
}

// ---------------------------------------------------------------------------
// Okada (1992) point source, DC3Dfortran.f90:2-607 with DCCON0 (:1236-1263),
// DCCON1 (:1267-1286), assign_alpha (:1400-1414).
// ---------------------------------------------------------------------------
static const double PI2 = 6.283185307179586e0;

static void dccon0(double dip, double *sd, double *cd) {
    const double P18 = PI2 / 360.0;
    *sd = sin(dip * P18);
    *cd = cos(dip * P18);
    if (fabs(*cd) < 1.0e-6) {
        *cd = 0.0;
        if (*sd > 0.0) *sd = 1.0;
        if (*sd < 0.0) *sd = -1.0;
    }
}

static void dccon1(double x, double y, double d, double sd, double cd, double *r, double *p,
                   double *q, double *s, double *t) {
    *p = y * cd + d * sd;
    *q = y * sd - d * cd;
    *s = *p * sd + *q * cd;
    *t = *p * cd - *q * sd;
    *r = sqrt(x * x + y * y + d * d);
}

static void ua0(double X, double Y, double D, double POT1, double POT2, double POT3, double POT4,
                double SD, double CD, const double ALP[5], double U[12]) {
    double DU[12];
    for (int i = 0; i < 12; ++i) { U[i] = 0.0; DU[i] = 0.0; }
    double R, P, Q, S, T;
    dccon1(X, Y, D, SD, CD, &R, &P, &Q, &S, &T);
    double S2D = 2.0 * SD * CD, C2D = CD * CD - SD * SD;
    double XY = X * Y, X2 = X * X, Y2 = Y * Y, D2 = D * D;
    double R2 = pow(R, 2.0), R3 = pow(R, 3.0), R5 = pow(R, 5.0);
    double QR = 3.0 * Q / R5, QRX = 5.0 * QR * X / R2;
    double A3 = 1.0 - 3.0 * X2 / R2, A5 = 1.0 - 5.0 * X2 / R2;
    double B3 = 1.0 - 3.0 * Y2 / R2, C3 = 1.0 - 3.0 * D2 / R2;
    double UY = SD - 5.0 * Y * Q / R2, UZ = CD + 5.0 * D * Q / R2;
    double VY = S - 5.0 * Y * P * Q / R2, VZ = T + 5.0 * D * P * Q / R2;
    double WY = UY + SD, WZ = UZ + CD;
    const double F3 = 3.0;
    if (POT1 != 0.0) {
        DU[0] = ALP[0] * Q / R3 + ALP[1] * X2 * QR;
        DU[1] = ALP[0] * X / R3 * SD + ALP[1] * XY * QR;
        DU[2] = -ALP[0] * X / R3 * CD + ALP[1] * X * D * QR;
        DU[3] = X * QR * (-ALP[0] + ALP[1] * (1.0 + A5));
        DU[4] = ALP[0] * A3 / R3 * SD + ALP[1] * Y * QR * A5;
        DU[5] = -ALP[0] * A3 / R3 * CD + ALP[1] * D * QR * A5;
        DU[6] = ALP[0] * (SD / R3 - Y * QR) + ALP[1] * F3 * X2 / R5 * UY;
        DU[7] = F3 * X / R5 * (-ALP[0] * Y * SD + ALP[1] * (Y * UY + Q));
        DU[8] = F3 * X / R5 * (ALP[0] * Y * CD + ALP[1] * D * UY);
        DU[9] = ALP[0] * (CD / R3 + D * QR) + ALP[1] * F3 * X2 / R5 * UZ;
        DU[10] = F3 * X / R5 * (ALP[0] * D * SD + ALP[1] * Y * UZ);
        DU[11] = F3 * X / R5 * (-ALP[0] * D * CD + ALP[1] * (D * UZ - Q));
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT1 / PI2 * DU[i];
    }
    if (POT2 != 0.0) {
        DU[0] = ALP[1] * X * P * QR;
        DU[1] = ALP[0] * S / R3 + ALP[1] * Y * P * QR;
        DU[2] = -ALP[0] * T / R3 + ALP[1] * D * P * QR;
        DU[3] = ALP[1] * P * QR * A5;
        DU[4] = -ALP[0] * F3 * X * S / R5 - ALP[1] * Y * P * QRX;
        DU[5] = ALP[0] * F3 * X * T / R5 - ALP[1] * D * P * QRX;
        DU[6] = ALP[1] * F3 * X / R5 * VY;
        DU[7] = ALP[0] * (S2D / R3 - F3 * Y * S / R5) + ALP[1] * (F3 * Y / R5 * VY + P * QR);
        DU[8] = -ALP[0] * (C2D / R3 - F3 * Y * T / R5) + ALP[1] * F3 * D / R5 * VY;
        DU[9] = ALP[1] * F3 * X / R5 * VZ;
        DU[10] = ALP[0] * (C2D / R3 + F3 * D * S / R5) + ALP[1] * F3 * Y / R5 * VZ;
        DU[11] = ALP[0] * (S2D / R3 - F3 * D * T / R5) + ALP[1] * (F3 * D / R5 * VZ - P * QR);
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT2 / PI2 * DU[i];
    }
    if (POT3 != 0.0) {
        DU[0] = ALP[0] * X / R3 - ALP[1] * X * Q * QR;
        DU[1] = ALP[0] * T / R3 - ALP[1] * Y * Q * QR;
        DU[2] = ALP[0] * S / R3 - ALP[1] * D * Q * QR;
        DU[3] = ALP[0] * A3 / R3 - ALP[1] * Q * QR * A5;
        DU[4] = -ALP[0] * F3 * X * T / R5 + ALP[1] * Y * Q * QRX;
        DU[5] = -ALP[0] * F3 * X * S / R5 + ALP[1] * D * Q * QRX;
        DU[6] = -ALP[0] * F3 * XY / R5 - ALP[1] * X * QR * WY;
        DU[7] = ALP[0] * (C2D / R3 - F3 * Y * T / R5) - ALP[1] * (Y * WY + Q) * QR;
        DU[8] = ALP[0] * (S2D / R3 - F3 * Y * S / R5) - ALP[1] * D * QR * WY;
        DU[9] = ALP[0] * F3 * X * D / R5 - ALP[1] * X * QR * WZ;
        DU[10] = -ALP[0] * (S2D / R3 - F3 * D * T / R5) - ALP[1] * Y * QR * WZ;
        DU[11] = ALP[0] * (C2D / R3 + F3 * D * S / R5) - ALP[1] * (D * WZ - Q) * QR;
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT3 / PI2 * DU[i];
    }
    if (POT4 != 0.0) {
        DU[0] = -ALP[0] * X / R3;
        DU[1] = -ALP[0] * Y / R3;
        DU[2] = -ALP[0] * D / R3;
        DU[3] = -ALP[0] * A3 / R3;
        DU[4] = ALP[0] * F3 * XY / R5;
        DU[5] = ALP[0] * F3 * X * D / R5;
        DU[6] = DU[4];
        DU[7] = -ALP[0] * B3 / R3;
        DU[8] = ALP[0] * F3 * Y * D / R5;
        DU[9] = -DU[5];
        DU[10] = -DU[8];
        DU[11] = ALP[0] * C3 / R3;
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT4 / PI2 * DU[i];
    }
}

static void ub0(double X, double Y, double D, double Z, double POT1, double POT2, double POT3,
                double POT4, double SD, double CD, const double ALP[5], double U[12]) {
    double DU[12];
    for (int i = 0; i < 12; ++i) { U[i] = 0.0; DU[i] = 0.0; }
    double R, P, Q, S, T;
    dccon1(X, Y, D, SD, CD, &R, &P, &Q, &S, &T);
    double XY = X * Y, X2 = X * X, Y2 = Y * Y, D2 = D * D;
    double R2 = pow(R, 2.0), R3 = pow(R, 3.0), R5 = pow(R, 5.0);
    double QR = 3.0 * Q / R5;
    double QRX = 5.0 * QR * X / R2;
    double A3 = 1.0 - 3.0 * X2 / R2, A5 = 1.0 - 5.0 * X2 / R2;
    double B3 = 1.0 - 3.0 * Y2 / R2, C3 = 1.0 - 3.0 * D2 / R2;
    double UY = SD - 5.0 * Y * Q / R2, UZ = CD + 5.0 * D * Q / R2;
    double VY = S - 5.0 * Y * P * Q / R2, VZ = T + 5.0 * D * P * Q / R2;
    double WY = UY + SD, WZ = UZ + CD;
    double C = D + Z, RD = R + D;
    double D12 = 1.0 / (R * RD * RD);
    double D32 = D12 * (2.0 * R + D) / R2;
    double D33 = D12 * (3.0 * R + D) / (R2 * RD);
    double D53 = D12 * (8.0 * R2 + 9.0 * R * D + 3.0 * D2) / (R2 * R2 * RD);
    double D54 = D12 * (5.0 * R2 + 4.0 * R * D + D2) / R3 * D12;
    double FI1 = Y * (D12 - X2 * D33);
    double FI2 = X * (D12 - Y2 * D33);
    double FI3 = X / R3 - FI2;
    double FI4 = -XY * D32;
    double FI5 = 1.0 / (R * RD) - X2 * D32;
    double FJ1 = -3.0 * XY * (D33 - X2 * D54);
    double FJ2 = 1.0 / R3 - 3.0 * D12 + 3.0 * X2 * Y2 * D54;
    double FJ3 = A3 / R3 - FJ2;
    double FJ4 = -3.0 * XY / R5 - FJ1;
    double FK1 = -Y * (D32 - X2 * D53);
    double FK2 = -X * (D32 - Y2 * D53);
    double FK3 = -3.0 * X * D / R5 - FK2;
    const double F3 = 3.0, F1 = 1.0;
    if (POT1 != 0.0) {
        DU[0] = -X2 * QR - ALP[2] * FI1 * SD;
        DU[1] = -XY * QR - ALP[2] * FI2 * SD;
        DU[2] = -C * X * QR - ALP[2] * FI4 * SD;
        DU[3] = -X * QR * (F1 + A5) - ALP[2] * FJ1 * SD;
        DU[4] = -Y * QR * A5 - ALP[2] * FJ2 * SD;
        DU[5] = -C * QR * A5 - ALP[2] * FK1 * SD;
        DU[6] = -F3 * X2 / R5 * UY - ALP[2] * FJ2 * SD;
        DU[7] = -F3 * XY / R5 * UY - X * QR - ALP[2] * FJ4 * SD;
        DU[8] = -F3 * C * X / R5 * UY - ALP[2] * FK2 * SD;
        DU[9] = -F3 * X2 / R5 * UZ + ALP[2] * FK1 * SD;
        DU[10] = -F3 * XY / R5 * UZ + ALP[2] * FK2 * SD;
        DU[11] = F3 * X / R5 * (-C * UZ + ALP[2] * Y * SD);
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT1 / PI2 * DU[i];
    }
    if (POT2 != 0.0) {
        DU[0] = -X * P * QR + ALP[2] * FI3 * SD * CD;
        DU[1] = -Y * P * QR + ALP[2] * FI1 * SD * CD;
        DU[2] = -C * P * QR + ALP[2] * FI5 * SD * CD;
        DU[3] = -P * QR * A5 + ALP[2] * FJ3 * SD * CD;
        DU[4] = Y * P * QRX + ALP[2] * FJ1 * SD * CD;
        DU[5] = C * P * QRX + ALP[2] * FK3 * SD * CD;
        DU[6] = -F3 * X / R5 * VY + ALP[2] * FJ1 * SD * CD;
        DU[7] = -F3 * Y / R5 * VY - P * QR + ALP[2] * FJ2 * SD * CD;
        DU[8] = -F3 * C / R5 * VY + ALP[2] * FK1 * SD * CD;
        DU[9] = -F3 * X / R5 * VZ - ALP[2] * FK3 * SD * CD;
        DU[10] = -F3 * Y / R5 * VZ - ALP[2] * FK1 * SD * CD;
        DU[11] = -F3 * C / R5 * VZ + ALP[2] * A3 / R3 * SD * CD;
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT2 / PI2 * DU[i];
    }
    if (POT3 != 0.0) {
        DU[0] = X * Q * QR - ALP[2] * FI3 * SD * SD;
        DU[1] = Y * Q * QR - ALP[2] * FI1 * SD * SD;
        DU[2] = C * Q * QR - ALP[2] * FI5 * SD * SD;
        DU[3] = Q * QR * A5 - ALP[2] * FJ3 * SD * SD;
        DU[4] = -Y * Q * QRX - ALP[2] * FJ1 * SD * SD;
        DU[5] = -C * Q * QRX - ALP[2] * FK3 * SD * SD;
        DU[6] = X * QR * WY - ALP[2] * FJ1 * SD * SD;
        DU[7] = QR * (Y * WY + Q) - ALP[2] * FJ2 * SD * SD;
        DU[8] = C * QR * WY - ALP[2] * FK1 * SD * SD;
        DU[9] = X * QR * WZ + ALP[2] * FK3 * SD * SD;
        DU[10] = Y * QR * WZ + ALP[2] * FK1 * SD * SD;
        DU[11] = C * QR * WZ - ALP[2] * A3 / R3 * SD * SD;
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT3 / PI2 * DU[i];
    }
    if (POT4 != 0.0) {
        DU[0] = ALP[2] * X / R3;
        DU[1] = ALP[2] * Y / R3;
        DU[2] = ALP[2] * D / R3;
        DU[3] = ALP[2] * A3 / R3;
        DU[4] = -ALP[2] * F3 * XY / R5;
        DU[5] = -ALP[2] * F3 * X * D / R5;
        DU[6] = DU[4];
        DU[7] = ALP[2] * B3 / R3;
        DU[8] = -ALP[2] * F3 * Y * D / R5;
        DU[9] = -DU[5];
        DU[10] = -DU[8];
        DU[11] = -ALP[2] * C3 / R3;
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT4 / PI2 * DU[i];
    }
}

static void uc0(double X, double Y, double D, double Z, double POT1, double POT2, double POT3,
                double POT4, double SD, double CD, const double ALP[5], double U[12]) {
    double DU[12];
    for (int i = 0; i < 12; ++i) { U[i] = 0.0; DU[i] = 0.0; }
    double R, P, Q, S, T;
    dccon1(X, Y, D, SD, CD, &R, &P, &Q, &S, &T);
    double XY = X * Y, X2 = X * X, Y2 = Y * Y, D2 = D * D;
    double R2 = pow(R, 2.0), R3 = pow(R, 3.0), R5 = pow(R, 5.0);
    double QR = 3.0 * Q / R5, QRX = 5.0 * QR * X / R2;
    double A3 = 1.0 - 3.0 * X2 / R2, A5 = 1.0 - 5.0 * X2 / R2;
    double C3 = 1.0 - 3.0 * D2 / R2;
    double S2D = 2.0 * SD * CD, C2D = CD * CD - SD * SD;
    double C = D + Z, Q2 = Q * Q, R7 = R5 * R2;
    double A7 = 1.0 - 7.0 * X2 / R2, B5 = 1.0 - 5.0 * Y2 / R2, B7 = 1.0 - 7.0 * Y2 / R2;
    double C5 = 1.0 - 5.0 * D2 / R2, C7 = 1.0 - 7.0 * D2 / R2, D7 = 2.0 - 7.0 * Q2 / R2;
    double QR5 = 5.0 * Q / R2, QR7 = 7.0 * Q / R2, DR5 = 5.0 * D / R2;
    const double F1 = 1.0, F2 = 2.0, F3 = 3.0, F5 = 5.0, F10 = 10.0, F15 = 15.0;
    (void)C3;
    if (POT1 != 0.0) {
        DU[0] = -ALP[3] * A3 / R3 * CD + ALP[4] * C * QR * A5;
        DU[1] = F3 * X / R5 * (ALP[3] * Y * CD + ALP[4] * C * (SD - Y * QR5));
        DU[2] = F3 * X / R5 * (-ALP[3] * Y * SD + ALP[4] * C * (CD + D * QR5));
        DU[3] = ALP[3] * F3 * X / R5 * (F2 + A5) * CD - ALP[4] * C * QRX * (F2 + A7);
        DU[4] = F3 / R5 * (ALP[3] * Y * A5 * CD + ALP[4] * C * (A5 * SD - Y * QR5 * A7));
        DU[5] = F3 / R5 * (-ALP[3] * Y * A5 * SD + ALP[4] * C * (A5 * CD + D * QR5 * A7));
        DU[6] = DU[4];
        DU[7] = F3 * X / R5 * (ALP[3] * B5 * CD - ALP[4] * F5 * C / R2 * (F2 * Y * SD + Q * B7));
        DU[8] = F3 * X / R5 * (-ALP[3] * B5 * SD + ALP[4] * F5 * C / R2 * (D * B7 * SD - Y * C7 * CD));
        DU[9] = F3 / R5 * (-ALP[3] * D * A5 * CD + ALP[4] * C * (A5 * CD + D * QR5 * A7));
        DU[10] = F15 * X / R7 * (ALP[3] * Y * D * CD + ALP[4] * C * (D * B7 * SD - Y * C7 * CD));
        DU[11] = F15 * X / R7 * (-ALP[3] * Y * D * SD + ALP[4] * C * (F2 * D * CD - Q * C7));
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT1 / PI2 * DU[i];
    }
    if (POT2 != 0.0) {
        DU[0] = ALP[3] * F3 * X * T / R5 - ALP[4] * C * P * QRX;
        DU[1] = -ALP[3] / R3 * (C2D - F3 * Y * T / R2) + ALP[4] * F3 * C / R5 * (S - Y * P * QR5);
        DU[2] = -ALP[3] * A3 / R3 * SD * CD + ALP[4] * F3 * C / R5 * (T + D * P * QR5);
        DU[3] = ALP[3] * F3 * T / R5 * A5 - ALP[4] * F5 * C * P * QR / R2 * A7;
        DU[4] = F3 * X / R5 * (ALP[3] * (C2D - F5 * Y * T / R2) - ALP[4] * F5 * C / R2 * (S - Y * P * QR7));
        DU[5] = F3 * X / R5 * (ALP[3] * (F2 + A5) * SD * CD - ALP[4] * F5 * C / R2 * (T + D * P * QR7));
        DU[6] = DU[4];
        DU[7] = F3 / R5 * (ALP[3] * (F2 * Y * C2D + T * B5) + ALP[4] * C * (S2D - F10 * Y * S / R2 - P * QR5 * B7));
        DU[8] = F3 / R5 * (ALP[3] * Y * A5 * SD * CD - ALP[4] * C * ((F3 + A5) * C2D + Y * P * DR5 * QR7));
        DU[9] = F3 * X / R5 * (-ALP[3] * (S2D - T * DR5) - ALP[4] * F5 * C / R2 * (T + D * P * QR7));
        DU[10] = F3 / R5 * (-ALP[3] * (D * B5 * C2D + Y * C5 * S2D) - ALP[4] * C * ((F3 + A5) * C2D + Y * P * DR5 * QR7));
        DU[11] = F3 / R5 * (-ALP[3] * D * A5 * SD * CD - ALP[4] * C * (S2D - F10 * D * T / R2 + P * QR5 * C7));
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT2 / PI2 * DU[i];
    }
    if (POT3 != 0.0) {
        DU[0] = F3 * X / R5 * (-ALP[3] * S + ALP[4] * (C * Q * QR5 - Z));
        DU[1] = ALP[3] / R3 * (S2D - F3 * Y * S / R2) + ALP[4] * F3 / R5 * (C * (T - Y + Y * Q * QR5) - Y * Z);
        DU[2] = -ALP[3] / R3 * (F1 - A3 * SD * SD) - ALP[4] * F3 / R5 * (C * (S - D + D * Q * QR5) - D * Z);
        DU[3] = -ALP[3] * F3 * S / R5 * A5 + ALP[4] * (C * QR * QR5 * A7 - F3 * Z / R5 * A5);
        DU[4] = F3 * X / R5 * (-ALP[3] * (S2D - F5 * Y * S / R2) - ALP[4] * F5 / R2 * (C * (T - Y + Y * Q * QR7) - Y * Z));
        DU[5] = F3 * X / R5 * (ALP[3] * (F1 - (F2 + A5) * SD * SD) + ALP[4] * F5 / R2 * (C * (S - D + D * Q * QR7) - D * Z));
        DU[6] = DU[4];
        DU[7] = F3 / R5 * (-ALP[3] * (F2 * Y * S2D + S * B5) - ALP[4] * (C * (F2 * SD * SD + F10 * Y * (T - Y) / R2 - Q * QR5 * B7) + Z * B5));
        DU[8] = F3 / R5 * (ALP[3] * Y * (F1 - A5 * SD * SD) + ALP[4] * (C * (F3 + A5) * S2D - Y * DR5 * (C * D7 + Z)));
        DU[9] = F3 * X / R5 * (-ALP[3] * (C2D + S * DR5) + ALP[4] * (F5 * C / R2 * (S - D + D * Q * QR7) - F1 - Z * DR5));
        DU[10] = F3 / R5 * (ALP[3] * (D * B5 * S2D - Y * C5 * C2D) + ALP[4] * (C * ((F3 + A5) * S2D - Y * DR5 * D7) - Y * (F1 + Z * DR5)));
        DU[11] = F3 / R5 * (-ALP[3] * D * (F1 - A5 * SD * SD) - ALP[4] * (C * (C2D + F10 * D * (S - D) / R2 - Q * QR5 * C7) + Z * (F1 + C5)));
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT3 / PI2 * DU[i];
    }
    if (POT4 != 0.0) {
        DU[0] = ALP[3] * F3 * X * D / R5;
        DU[1] = ALP[3] * F3 * Y * D / R5;
        DU[2] = ALP[3] * (1.0 - 3.0 * D2 / R2) / R3;
        DU[3] = ALP[3] * F3 * D / R5 * A5;
        DU[4] = -ALP[3] * F15 * XY * D / R7;
        DU[5] = -ALP[3] * F3 * X / R5 * C5;
        DU[6] = DU[4];
        DU[7] = ALP[3] * F3 * D / R5 * B5;
        DU[8] = -ALP[3] * F3 * Y / R5 * C5;
        DU[9] = DU[5];
        DU[10] = DU[8];
        DU[11] = ALP[3] * F3 * D / R5 * (F2 + C5);
        for (int i = 0; i < 12; ++i) U[i] = U[i] + POT4 / PI2 * DU[i];
    }
}

// DC3D0 (DC3Dfortran.f90:2-118)
extern "C" void orc_dc3d0(double alpha, double x, double y, double z, double depth, double dip,
                          double pot1, double pot2, double pot3, double pot4, double u[12],
                          int32_t *iret) {
    double U[12], DUA[12], DUB[12], DUC[12];
    for (int i = 0; i < 12; ++i) { U[i] = 0.0; DUA[i] = 0.0; DUB[i] = 0.0; DUC[i] = 0.0; }
    for (int i = 0; i < 12; ++i) u[i] = 0.0;
    double XX = x, YY = y, ZZ = z, DD = depth + z;
    // depth < 0: early return with zero output; IRET is left unset by the
    // reference (DC3Dfortran.f90:67-70); here it reads -1.
    if (depth < 0.0) { *iret = -1; return; }
    const double EPS = 1.0e-6;
    if (fabs(XX) < EPS) XX = 0.0;
    if (fabs(YY) < EPS) YY = 0.0;
    if (fabs(DD) < EPS) DD = 0.0;
    *iret = 0;
    if (z > 0.0) { *iret = 2; return; }
    double R = sqrt(XX * XX + YY * YY + DD * DD);
    if (R == 0.0) { *iret = 1; return; }
    double ALP[5] = {(1.0 - alpha) / 2.0, alpha / 2.0, (1.0 - alpha) / alpha, 1.0 - alpha, alpha};
    double SD, CD;
    dccon0(dip, &SD, &CD);
    ua0(XX, YY, DD, pot1, pot2, pot3, pot4, SD, CD, ALP, DUA);
    for (int i = 0; i < 12; ++i) {
        if (i < 9) U[i] = U[i] - DUA[i];
        else U[i] = U[i] + DUA[i];
    }
    DD = depth - z;
    ua0(XX, YY, DD, pot1, pot2, pot3, pot4, SD, CD, ALP, DUA);
    ub0(XX, YY, DD, ZZ, pot1, pot2, pot3, pot4, SD, CD, ALP, DUB);
    uc0(XX, YY, DD, ZZ, pot1, pot2, pot3, pot4, SD, CD, ALP, DUC);
    for (int i = 0; i < 12; ++i) {
        double DU = DUA[i] + DUB[i] + ZZ * DUC[i];
        if (i >= 9) DU = DU + DUC[i - 9];
        U[i] = U[i] + DU;
    }
    for (int i = 0; i < 12; ++i) u[i] = U[i];
}

// call_dc3d0 (gfunc.f90:65-100)
static void call_dc3d0(double xsource, double ysource, double zsource, double xobs, double yobs,
                       double uxi, double ueta, double dip, double area, double strike,
                       double alpha, double uret[3]) {
    double M_PI_ = 2.0 * asin(1.0);
    double strike_rad = strike / 180.0 * M_PI_;
    double x = sin(strike_rad) * (xobs - xsource) + cos(strike_rad) * (yobs - ysource);
    double y = -cos(strike_rad) * (xobs - xsource) + sin(strike_rad) * (yobs - ysource);
    double z = 0.0;
    double depth = -(zsource);
    double pot1 = uxi * area, pot2 = ueta * area;
    double u[12];
    int32_t iret;
    orc_dc3d0(alpha, x, y, z, depth, dip, pot1, pot2, 0.0, 0.0, u, &iret);
    double ux_rot = sin(strike_rad) * u[0] - cos(strike_rad) * u[1];
    double uy_rot = cos(strike_rad) * u[0] + sin(strike_rad) * u[1];
    uret[0] = 100.0 * ux_rot;
    uret[1] = 100.0 * uy_rot;
    uret[2] = 100.0 * u[2];
}

// ---------------------------------------------------------------------------
// Geometry and discretisation (init.f90:121-293, main.f90:209-246)
// ---------------------------------------------------------------------------
struct Plane { double xf, yf, zf, strike, dip, lxi, leta; int nxi, neta; };

static int ndim_fault_of(const orc_setup *s) {
    if (s->layout == 0) return 3 * s->nplane + 3;
    if (s->layout == 1) return 2 * s->nplane + 4;
    return s->rect_hyper ? 10 : 8;
}

// get_geometry (init.f90:121-173) + fault centre (gfunc.f90:283-296); the
// buried-rectangle layout maps theta straight onto the same plane fields.
static void planes_of(const orc_setup *s, const double *theta, std::vector<Plane> &pl) {
    pl.resize(s->nplane);
    if (s->layout == 2) {
        double pi = 4.0 * atan(1.0);
        Plane &p = pl[0];
        double dip_rad = theta[6] * pi / 180.0;
        p.xf = theta[0]; p.yf = theta[1];
        p.zf = -(theta[2] + theta[4] / 2.0 * sin(dip_rad));
        p.lxi = theta[3]; p.leta = theta[4];
        p.strike = theta[5]; p.dip = theta[6];
        p.nxi = s->nxi[0]; p.neta = s->neta[0];
        return;
    }
    double pi = 4.0 * atan(1.0);
    double ymin = theta[0], ymax = theta[1];
    int nplane = s->nplane;
    for (int ip = 1; ip <= nplane; ++ip) {
        double xl, yl, xr, yr, dip;
        if (s->layout == 1) {
            if (ip == 1) { xl = s->xmin; yl = ymin; } else { xl = s->xbend[ip - 2]; yl = theta[ip]; }
            if (ip == nplane) { xr = s->xmax; yr = ymax; } else { xr = s->xbend[ip - 1]; yr = theta[ip + 1]; }
            dip = theta[nplane + ip];
        } else {
            if (ip == 1) { xl = s->xmin; yl = ymin; } else { xl = theta[2 * ip - 2]; yl = theta[2 * ip - 1]; }
            if (ip == nplane) { xr = s->xmax; yr = ymax; } else { xr = theta[2 * ip]; yr = theta[2 * ip + 1]; }
            dip = theta[2 * nplane + ip - 1];
        }
        double dip_rad = dip * pi / 180.0;
        double lxi = sqrt((xr - xl) * (xr - xl) + (yr - yl) * (yr - yl));
        double leta = -s->zmin / sin(dip_rad);
        double strike_rad = atan2(xr - xl, yr - yl);
        double strike = strike_rad / pi * 180.0;
        Plane &p = pl[ip - 1];
        p.xf = (xl + xr) / 2.0 - (s->zmin * cos(strike_rad)) / (2.0 * tan(dip_rad));
        p.yf = (yl + yr) / 2.0 + (s->zmin * sin(strike_rad)) / (2.0 * tan(dip_rad));
        p.zf = s->zmin / 2.0;
        p.strike = strike; p.dip = dip; p.lxi = lxi; p.leta = leta;
        p.nxi = s->nxi[ip - 1]; p.neta = s->neta[ip - 1];
    }
}

extern "C" void orc_hyper(const orc_setup *s, const double *theta, double *log_alpha2,
                          double *log_sigma_sar2, double *log_sigma_gnss2) {
    // get_sigma (init.f90:175-196)
    int n = s->nplane;
    if (s->layout == 2) {
        *log_alpha2 = theta[7];
        *log_sigma_sar2 = s->rect_hyper ? theta[8] : 0.0;
        *log_sigma_gnss2 = s->rect_hyper ? theta[9] : 0.0;
    } else if (s->layout == 1) {
        *log_alpha2 = theta[2 * n + 1]; *log_sigma_sar2 = theta[2 * n + 2]; *log_sigma_gnss2 = theta[2 * n + 3];
    } else {
        *log_alpha2 = theta[3 * n]; *log_sigma_sar2 = theta[3 * n + 1]; *log_sigma_gnss2 = theta[3 * n + 2];
    }
}

struct Mesh {
    int nnode, npatch, ndof, D;
    std::vector<double> coor;          // [nnode][2] (xi, eta)
    std::vector<int> cny;              // [npatch][4] node ids
    std::vector<int> n2e_val, n2e_size; // [nnode][4], [nnode]
    std::vector<int> id_dof;           // [ndof] node ids
    std::vector<int> plane_of_patch;
    std::vector<int> ndof_index;       // per plane, nplane+1
};

// discretize_fault (init.f90:198-293) with DOF counts of main.f90:209-238
static void discretize(const orc_setup *s, const std::vector<Plane> &pl, Mesh &m) {
    int nplane = s->nplane;
    int nn = 0, np = 0;
    for (int ip = 0; ip < nplane; ++ip) { nn += (pl[ip].nxi + 1) * (pl[ip].neta + 1); np += pl[ip].nxi * pl[ip].neta; }
    m.nnode = nn; m.npatch = np;
    m.coor.assign(2 * nn, 0.0);
    m.cny.assign(4 * np, 0);
    m.n2e_val.assign(4 * nn, -1);
    m.n2e_size.assign(nn, 0);
    m.id_dof.clear();
    m.plane_of_patch.assign(np, 0);
    m.ndof_index.assign(nplane + 1, 0);
    int off_node = 0, off_patch = 0;
    for (int ip = 0; ip < nplane; ++ip) {
        int nxi = pl[ip].nxi, neta = pl[ip].neta;
        double dxi = pl[ip].lxi / nxi, deta = pl[ip].leta / neta;
        m.ndof_index[ip] = (int)m.id_dof.size();
        for (int j = 1; j <= neta + 1; ++j)
            for (int i = 1; i <= nxi + 1; ++i) {
                int node = i + (nxi + 1) * (j - 1) + off_node - 1;
                m.coor[2 * node] = (i - 1) * dxi - pl[ip].lxi / 2.0;
                m.coor[2 * node + 1] = (j - 1) * deta - pl[ip].leta / 2.0;
                if (j == 1) continue;
                if (ip == 0 && i == 1) continue;
                if (ip == nplane - 1 && i == nxi + 1) continue;
                m.id_dof.push_back(node);
            }
        for (int j = 1; j <= neta; ++j)
            for (int i = 1; i <= nxi; ++i) {
                int patch = off_patch + i + nxi * (j - 1) - 1;
                int n1 = i + (nxi + 1) * (j - 1) + off_node - 1;
                int c[4] = {n1, n1 + 1, n1 + 1 + nxi + 1, n1 + nxi + 1};
                for (int k = 0; k < 4; ++k) {
                    m.cny[4 * patch + k] = c[k];
                    int sz = m.n2e_size[c[k]]++;
                    m.n2e_val[4 * c[k] + sz] = patch;
                }
                m.plane_of_patch[patch] = ip;
            }
        off_patch += nxi * neta;
        off_node += (nxi + 1) * (neta + 1);
    }
    m.ndof_index[nplane] = (int)m.id_dof.size();
    m.ndof = (int)m.id_dof.size();
    m.D = (s->basis == 0) ? 2 * m.ndof : 2 * m.npatch;
}

extern "C" int orc_dims(const orc_setup *s, orc_dims_t *out) {
    int nn = 0, np = 0, nd = 0;
    for (int ip = 0; ip < s->nplane; ++ip) {
        int nxi = s->nxi[ip], neta = s->neta[ip];
        nn += (nxi + 1) * (neta + 1);
        np += nxi * neta;
        int d = (nxi + 1) * (neta + 1) - (nxi + 1);
        if (ip == 0) d -= neta;
        if (ip == s->nplane - 1) d -= neta;
        nd += d;
    }
    out->ndim_fault = ndim_fault_of(s);
    out->nnode = nn; out->npatch = np; out->ndof = nd;
    out->D = s->basis == 0 ? 2 * nd : 2 * np;
    out->nrow_l = s->basis == 0 ? 2 * nn : 2 * np;
    return 0;
}

// point_cloud (main.f90:666-781).  The reference reads each plane's centre,
// strike, dip and size from an 8-entries-per-plane theta that none of its
// get_geometry layouts produces; the plane record of calc_greens_func
// (gfunc.f90:283-296) is the one that describes the sampled fault.
extern "C" int orc_point_cloud(const orc_setup *s, const double *theta, const double *slip, int32_t nr,
                               double *points) {
    std::vector<Plane> pl;
    planes_of(s, theta, pl);
    Mesh m;
    discretize(s, pl, m);
    double pi = 4.0 * atan(1.0);
    std::vector<double> rv(nr);
    for (int ir = 1; ir <= nr; ++ir) rv[ir - 1] = -1.0 + 1.0 / (double)nr + (ir - 1) * 2.0 / (double)nr;
    int off_patch = 0;
    for (int ip = 0; ip < s->nplane; ++ip) {
        double strike_rad = pl[ip].strike * pi / 180.0, dip_rad = pl[ip].dip * pi / 180.0;
        for (int ie = off_patch; ie < off_patch + pl[ip].nxi * pl[ip].neta; ++ie) {
            double xin[4], etan[4], uxn[4], uen[4];
            for (int k = 0; k < 4; ++k) {
                int node = m.cny[4 * ie + k];
                xin[k] = m.coor[2 * node];
                etan[k] = m.coor[2 * node + 1];
                uxn[k] = s->basis == 0 ? slip[2 * node] : slip[2 * ie];
                uen[k] = s->basis == 0 ? slip[2 * node + 1] : slip[2 * ie + 1];
            }
            for (int ir1 = 0; ir1 < nr; ++ir1)
                for (int ir2 = 0; ir2 < nr; ++ir2) {
                    double r1 = rv[ir1], r2 = rv[ir2];
                    double nv[4] = {(1.0 - r1) * (1.0 - r2) / 4.0, (1.0 + r1) * (1.0 - r2) / 4.0,
                                    (1.0 + r1) * (1.0 + r2) / 4.0, (1.0 - r1) * (1.0 + r2) / 4.0};
                    double xi = 0.0, eta = 0.0, uxi = 0.0, ueta = 0.0;
                    for (int k = 0; k < 4; ++k) {
                        xi = xi + nv[k] * xin[k];
                        eta = eta + nv[k] * etan[k];
                        uxi = uxi + nv[k] * uxn[k];
                        ueta = ueta + nv[k] * uen[k];
                    }
                    double *o = points + (((size_t)ie * nr + ir1) * nr + ir2) * 6;
                    o[0] = pl[ip].xf - eta * cos(dip_rad) * cos(strike_rad) + xi * sin(strike_rad);
                    o[1] = pl[ip].yf + eta * cos(dip_rad) * sin(strike_rad) + xi * cos(strike_rad);
                    o[2] = pl[ip].zf + eta * sin(dip_rad);
                    o[3] = uxi;
                    o[4] = ueta;
                    o[5] = sqrt(uxi * uxi + ueta * ueta);
                }
        }
        off_patch += pl[ip].nxi * pl[ip].neta;
    }
    return 0;
}

extern "C" void orc_plane_params(const orc_setup *s, const double *theta, double *out) {
    std::vector<Plane> pl;
    planes_of(s, theta, pl);
    for (int ip = 0; ip < s->nplane; ++ip) {
        out[7 * ip + 0] = pl[ip].xf; out[7 * ip + 1] = pl[ip].yf; out[7 * ip + 2] = pl[ip].zf;
        out[7 * ip + 3] = pl[ip].strike; out[7 * ip + 4] = pl[ip].dip;
        out[7 * ip + 5] = pl[ip].lxi; out[7 * ip + 6] = pl[ip].leta;
    }
}

// Gauss-Legendre nodes/weights on [-1,1]; order 2 uses the reference's
// literal +-1/sqrt(3) (gfunc.f90:125-128).
static void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0); w.assign(n, 0.0);
    if (n == 2) { x[0] = -1.0 / sqrt(3.0); x[1] = 1.0 / sqrt(3.0); w[0] = w[1] = 1.0; return; }
    double pi = 4.0 * atan(1.0);
    for (int i = 0; i < n; ++i) {
        long double z = cosl((long double)pi * (i + 0.75L) / (n + 0.5L)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1, p2 = 0;
            for (int k = 1; k <= n; ++k) { long double p3 = p2; p2 = p1; p1 = ((2 * k - 1) * z * p2 - (k - 1) * p3) / k; }
            pp = n * (z * p1 - p2) / (z * z - 1);
            long double z1 = z;
            z = z1 - p1 / pp;
            if (fabsl(z - z1) < 1e-19L) break;
        }
        x[n - 1 - i] = (double)z;     // ascending
        w[n - 1 - i] = (double)(2 / ((1 - z * z) * pp * pp));
    }
}

// calc_responce + calc_responce_dist + calc_greens_func (gfunc.f90:102-348).
// basis 0 is the reference's nodal loop (per DOF node, per direction, per
// station, per touching patch, per Gauss point); basis 1 is the
// patch-constant variant with the same source placement and conventions
// (strike unit slip -1, dip unit slip +1, gfunc.f90:13-18).
static void greens_impl(const orc_setup *s, const std::vector<Plane> &pl, const Mesh &m, double *gmat) {
    int nobs = s->nobs, D = m.D;
    std::vector<double> r, wq;
    gauss_legendre(s->nquad, r, wq);
    int nq = s->nquad;
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < nobs; ++i) gmat[(size_t)j * nobs + i] = 0.0;
    std::vector<double> resp(3 * (size_t)nobs);
    double M_PI_ = 2.0 * asin(1.0);

    auto one_station = [&](double xobs, double yobs, const Plane &p, const int *targets, int ntarget,
                           int unit_node, int dir, double uobs[3]) {
        double dip_rad = p.dip / 180.0 * M_PI_;
        double strike_rad = p.strike / 180.0 * M_PI_;
        uobs[0] = uobs[1] = uobs[2] = 0.0;
        for (int it = 0; it < ntarget; ++it) {
            int ie = targets[it];
            double xin[4], etn[4], uxin[4], uetn[4];
            for (int k = 0; k < 4; ++k) {
                int jn = m.cny[4 * ie + k];
                xin[k] = m.coor[2 * jn];
                etn[k] = m.coor[2 * jn + 1];
                double sl = 0.0;
                if (unit_node < 0 || jn == unit_node) sl = 1.0;
                uxin[k] = (dir == 1) ? -sl : 0.0;
                uetn[k] = (dir == 2) ? sl : 0.0;
            }
            double area = (xin[1] - xin[0]) * (etn[2] - etn[1]);
            for (int a = 0; a < nq; ++a) {
                double r1 = r[a];
                for (int b = 0; b < nq; ++b) {
                    double r2 = r[b];
                    double nv[4] = {(1.0 - r1) * (1.0 - r2) / 4.0, (1.0 + r1) * (1.0 - r2) / 4.0,
                                    (1.0 + r1) * (1.0 + r2) / 4.0, (1.0 - r1) * (1.0 + r2) / 4.0};
                    double xi = 0.0, eta = 0.0, uxi = 0.0, ueta = 0.0;
                    for (int k = 0; k < 4; ++k) {
                        xi = xi + nv[k] * xin[k];
                        eta = eta + nv[k] * etn[k];
                        uxi = uxi + nv[k] * uxin[k];
                        ueta = ueta + nv[k] * uetn[k];
                    }
                    double xs = p.xf - eta * cos(dip_rad) * cos(strike_rad) + xi * sin(strike_rad);
                    double ys = p.yf + eta * cos(dip_rad) * sin(strike_rad) + xi * cos(strike_rad);
                    double zs = p.zf + eta * sin(dip_rad);
                    double wgt = (nq == 2) ? area / 4.0 : area * wq[a] * wq[b] / 4.0;
                    double uret[3];
                    call_dc3d0(xs, ys, zs, xobs, yobs, uxi, ueta, p.dip, wgt, p.strike, s->alpha, uret);
                    for (int d = 0; d < 3; ++d) uobs[d] = uobs[d] + uret[d];
                }
            }
        }
    };

    auto column = [&](const Plane &p, const int *targets, int ntarget, int unit_node, int dir, int col) {
        double uobs[3];
        for (int io = 0; io < s->nsar_total; ++io) {
            one_station(s->obs_points[2 * io], s->obs_points[2 * io + 1], p, targets, ntarget, unit_node, dir, uobs);
            for (int d = 0; d < 3; ++d) resp[3 * io + d] = uobs[d];
        }
        for (int ig = 0; ig < s->ngnss; ++ig) {
            int row = s->nsar_total + 3 * ig;
            one_station(s->obs_points[2 * row], s->obs_points[2 * row + 1], p, targets, ntarget, unit_node, dir, uobs);
            for (int d = 0; d < 3; ++d) {
                resp[3 * row + d] = uobs[d];
                resp[3 * (row + 1) + d] = uobs[d];
                resp[3 * (row + 2) + d] = uobs[d];
            }
        }
        double *g = gmat + (size_t)col * nobs;
        for (int io = 0; io < nobs; ++io)
            for (int d = 0; d < 3; ++d) g[io] = g[io] + resp[3 * io + d] * s->obs_unitvec[3 * io + d];
    };

    if (s->basis == 0) {
        for (int ip = 0; ip < s->nplane; ++ip)
            for (int idof = m.ndof_index[ip]; idof < m.ndof_index[ip + 1]; ++idof) {
                int inode = m.id_dof[idof];
                int targets[4];
                int nt = m.n2e_size[inode];
                for (int t = 0; t < nt; ++t) targets[t] = m.n2e_val[4 * inode + t];
                for (int dir = 1; dir <= 2; ++dir) column(pl[ip], targets, nt, inode, dir, 2 * idof + dir - 1);
            }
    } else {
        for (int ie = 0; ie < m.npatch; ++ie) {
            int targets[1] = {ie};
            for (int dir = 1; dir <= 2; ++dir) column(pl[m.plane_of_patch[ie]], targets, 1, -1, dir, 2 * ie + dir - 1);
        }
    }
}

extern "C" int orc_greens(const orc_setup *s, const double *theta, double *gmat) {
    std::vector<Plane> pl;
    planes_of(s, theta, pl);
    Mesh m;
    discretize(s, pl, m);
    greens_impl(s, pl, m, gmat);
    return 0;
}

extern "C" int orc_greens_batch(const orc_setup *s, int32_t n, const double *theta, double *gmat,
                                int32_t nthreads) {
    orc_dims_t dm;
    orc_dims(s, &dm);
    size_t gsz = (size_t)s->nobs * dm.D;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int t = 0; t < n; ++t) orc_greens(s, theta + (size_t)t * dm.ndim_fault, gmat + (size_t)t * gsz);
    return 0;
}

// gen_laplacian (init.f90:295-474) on a (npx x npy) point grid; gen_sparse_lmat
// (:476-521); calc_ll (:523-541).  Basis 1 applies the same stencil to the
// patch-centre grid with every patch a degree of freedom.
struct Lap {
    int nrow, D;
    std::vector<int> lidx, ltidx;      // [nrow][9], [D][9] (0-based columns)
    std::vector<double> lval, ltval, ll;
};

static void laplacian_impl(const orc_setup *s, const std::vector<Plane> &pl, const Mesh &m, Lap &lp) {
    int npt = 0;
    std::vector<int> px(s->nplane), py(s->nplane);
    for (int ip = 0; ip < s->nplane; ++ip) {
        px[ip] = (s->basis == 0) ? pl[ip].nxi + 1 : pl[ip].nxi;
        py[ip] = (s->basis == 0) ? pl[ip].neta + 1 : pl[ip].neta;
        npt += px[ip] * py[ip];
    }
    std::vector<double> luni((size_t)npt * npt, 0.0);
    auto L = [&](int i, int j) -> double & { return luni[(size_t)j * npt + i]; };
    int offset = 0;
    for (int ip = 0; ip < s->nplane; ++ip) {
        double dxi = pl[ip].lxi / pl[ip].nxi, deta = pl[ip].leta / pl[ip].neta;
        int nx = px[ip] - 1, ny = py[ip] - 1;   // reference's nxi, neta
        for (int inode1 = offset + 1; inode1 <= offset + (nx + 1) * (ny + 1); ++inode1) {
            int k = (inode1 - 1 - offset) % (nx + 1) + 1;
            int l = (inode1 - 1 - offset) / (nx + 1) + 1;
            int in = inode1 - 1;
            int W = nx + 1;
            double cxx = 1.0 / (dxi * dxi), cyy = 1.0 / (deta * deta), cxy = 1.0 / (4.0 * dxi * deta);
            L(in, in) = L(in, in) - 2.0 / pow(dxi, 2);
            if (k == nx + 1) L(in, in - 1) = L(in, in - 1) + 1.0 / pow(dxi, 2);
            else L(in, in + 1) = L(in, in + 1) + 1.0 / pow(dxi, 2);
            if (k == 1) L(in, in + 1) = L(in, in + 1) + 1.0 / pow(dxi, 2);
            else L(in, in - 1) = L(in, in - 1) + 1.0 / pow(dxi, 2);
            if (l == ny + 1) L(in, in - W) = L(in, in - W) + 1.0 / pow(deta, 2);
            else L(in, in + W) = L(in, in + W) + 1.0 / pow(deta, 2);
            if (l == 1) L(in, in + W) = L(in, in + W) + 1.0 / pow(deta, 2);
            else L(in, in - W) = L(in, in - W) + 1.0 / pow(deta, 2);
            (void)cxx; (void)cyy; (void)cxy;
            double c = 1.0 / (4.0 * dxi * deta);
            if (k == nx + 1 && l == ny + 1) L(in, in - W - 1) = L(in, in - W - 1) + c;
            else if (k == nx + 1) L(in, in + W - 1) = L(in, in + W - 1) + c;
            else if (l == ny + 1) L(in, in - W + 1) = L(in, in - W + 1) + c;
            else L(in, in + W + 1) = L(in, in + W + 1) + c;
            if (k == 1 && l == ny + 1) L(in, in - W + 1) = L(in, in - W + 1) - c;
            else if (k == 1) L(in, in + W + 1) = L(in, in + W + 1) - c;
            else if (l == ny + 1) L(in, in - W - 1) = L(in, in - W - 1) - c;
            else L(in, in + W - 1) = L(in, in + W - 1) - c;
            if (k == 1 && l == 1) L(in, in + W + 1) = L(in, in + W + 1) + c;
            else if (k == 1) L(in, in - W + 1) = L(in, in - W + 1) + c;
            else if (l == 1) L(in, in + W - 1) = L(in, in + W - 1) + c;
            else L(in, in - W - 1) = L(in, in - W - 1) + c;
            if (k == nx + 1 && l == 1) L(in, in + W - 1) = L(in, in + W - 1) - c;
            else if (k == nx + 1) L(in, in - W - 1) = L(in, in - W - 1) - c;
            else if (l == 1) L(in, in + W + 1) = L(in, in + W + 1) - c;
            else L(in, in - W + 1) = L(in, in - W + 1) - c;
        }
        offset += (nx + 1) * (ny + 1);
    }
    // expansion to two components over the DOF columns
    std::vector<int> dofs;
    if (s->basis == 0) dofs = m.id_dof;
    else { dofs.resize(npt); for (int i = 0; i < npt; ++i) dofs[i] = i; }
    int nd = (int)dofs.size();
    int nrow = 2 * npt, D = 2 * nd;
    std::vector<double> lmat((size_t)nrow * D, 0.0);
    for (int in = 0; in < npt; ++in)
        for (int id = 0; id < nd; ++id) {
            int jn = dofs[id];
            lmat[(size_t)(2 * id) * nrow + 2 * in] = L(in, jn);
            lmat[(size_t)(2 * id + 1) * nrow + 2 * in + 1] = L(in, jn);
        }
    lp.nrow = nrow; lp.D = D;
    lp.lidx.assign((size_t)nrow * 9, 0); lp.lval.assign((size_t)nrow * 9, 0.0);
    lp.ltidx.assign((size_t)D * 9, 0); lp.ltval.assign((size_t)D * 9, 0.0);
    for (int i = 0; i < nrow; ++i) {
        int cnt = 0;
        for (int j = 0; j < D; ++j) {
            double v = lmat[(size_t)j * nrow + i];
            if (fabs(v) > 1e-8) { lp.lidx[9 * i + cnt] = j; lp.lval[9 * i + cnt] = v; ++cnt; }
        }
        while (cnt < 9) { lp.lidx[9 * i + cnt] = 0; lp.lval[9 * i + cnt] = 0.0; ++cnt; }
    }
    for (int i = 0; i < D; ++i) {
        int cnt = 0;
        for (int j = 0; j < nrow; ++j) {
            double v = lmat[(size_t)i * nrow + j];
            if (fabs(v) > 1e-8) { lp.ltidx[9 * i + cnt] = j; lp.ltval[9 * i + cnt] = v; ++cnt; }
        }
        while (cnt < 9) { lp.ltidx[9 * i + cnt] = 0; lp.ltval[9 * i + cnt] = 0.0; ++cnt; }
    }
    lp.ll.assign((size_t)D * D, 0.0);
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
            double t = 0.0;
            for (int k = 0; k < nrow; ++k) t += lmat[(size_t)i * nrow + k] * lmat[(size_t)j * nrow + k];
            lp.ll[(size_t)j * D + i] = t;
        }
}

extern "C" int orc_laplacian(const orc_setup *s, const double *theta, int32_t *lidx, double *lval,
                             int32_t *ltidx, double *ltval, double *llmat) {
    std::vector<Plane> pl;
    planes_of(s, theta, pl);
    Mesh m;
    discretize(s, pl, m);
    Lap lp;
    laplacian_impl(s, pl, m, lp);
    if (lidx) for (size_t i = 0; i < lp.lidx.size(); ++i) { lidx[i] = lp.lidx[i]; lval[i] = lp.lval[i]; }
    if (ltidx) for (size_t i = 0; i < lp.ltidx.size(); ++i) { ltidx[i] = lp.ltidx[i]; ltval[i] = lp.ltval[i]; }
    if (llmat) memcpy(llmat, lp.ll.data(), lp.ll.size() * sizeof(double));
    return lp.nrow;
}

// calc_sigma_sar_mat (init.f90:82-119): exponential covariance per path,
// inverted by LU with partial pivoting (dgetrf/dgetri).
extern "C" void orc_sigma_sar_inv(int32_t nobs, int32_t npath, const int32_t *nsar_index, const double *obs_points,
                                  const double *obs_sigma, double corr_len, double *out) {
    size_t off = 0;
    for (int p = 0; p < npath; ++p) {
        int n = nsar_index[p + 1] - nsar_index[p], st = nsar_index[p];
        std::vector<double> a((size_t)n * n), inv((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i) {
            double xi = obs_points[2 * (st + i)], yi = obs_points[2 * (st + i) + 1];
            for (int j = 0; j < n; ++j) {
                double xj = obs_points[2 * (st + j)], yj = obs_points[2 * (st + j) + 1];
                double dist = sqrt((xi - xj) * (xi - xj) + (yi - yj) * (yi - yj));
                // the reference reads obs_sigma(nsar_index(ipath) + iobs) with a
                // 1-based path start, i.e. one row past the point's own row
                // (init.f90:106-108); restated as written, clamped at the last row.
                int ri = std::min(st + i + 1, nobs - 1);
                int rj = std::min(st + j + 1, nobs - 1);
                a[(size_t)j * n + i] = obs_sigma[ri] * obs_sigma[rj] * exp(-dist / corr_len);
            }
        }
        for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
        // Gauss-Jordan with partial pivoting on [a | I]
        for (int c = 0; c < n; ++c) {
            int piv = c;
            for (int r = c + 1; r < n; ++r) if (fabs(a[(size_t)c * n + r]) > fabs(a[(size_t)c * n + piv])) piv = r;
            if (piv != c)
                for (int k = 0; k < n; ++k) {
                    std::swap(a[(size_t)k * n + c], a[(size_t)k * n + piv]);
                    std::swap(inv[(size_t)k * n + c], inv[(size_t)k * n + piv]);
                }
            double d = a[(size_t)c * n + c];
            for (int k = 0; k < n; ++k) { a[(size_t)k * n + c] /= d; inv[(size_t)k * n + c] /= d; }
            // eliminate column c from every other row: row r -= f_r row c, with
            // f_r = a(r, c) read before the update; columns outer, rows inner
            // (contiguous), each element updated exactly as row by row
            std::vector<double> f(a.begin() + (size_t)c * n, a.begin() + (size_t)(c + 1) * n);
            for (int k = 0; k < n; ++k) {
                const double akc = a[(size_t)k * n + c], ikc = inv[(size_t)k * n + c];
                double *ak = &a[(size_t)k * n], *ik = &inv[(size_t)k * n];
                for (int r = 0; r < n; ++r) {
                    if (r == c || f[r] == 0.0) continue;
                    ak[r] -= f[r] * akc;
                    ik[r] -= f[r] * ikc;
                }
            }
        }
        memcpy(out + off, inv.data(), inv.size() * sizeof(double));
        off += (size_t)n * n;
    }
}

// slip_calc_gsd_gsg (smc_slip.f90:1347-1443)
extern "C" void orc_gram(const orc_setup *s, const double *gmat, double sigma_sar2, double sigma_gnss2,
                         double *gsgmat, double *gsdvec, double *dsd) {
    int nobs = s->nobs;
    orc_dims_t dm;
    orc_dims(s, &dm);
    int D = dm.D;
    std::vector<double> sdvec(nobs, 0.0), gts((size_t)D * nobs, 0.0);
    size_t off = 0;
    for (int p = 0; p < s->npath; ++p) {
        int st = s->nsar_index[p], n = s->nsar_index[p + 1] - st;
        const double *Si = s->sigma_sar_inv + off;
        for (int j = 0; j < n; ++j) {      // dgemv('n'): y += A(:,j) * (alpha*x(j))
            double t = (1.0 / sigma_sar2) * s->dvec[st + j];
            for (int i = 0; i < n; ++i) sdvec[st + i] += t * Si[(size_t)j * n + i];
        }
        for (int j = 0; j < n; ++j)        // dgemm('t','n'): gts(:, st+j) = alpha * Gp^T Sinv(:,j)
            for (int i = 0; i < D; ++i) {
                double t = 0.0;
                for (int l = 0; l < n; ++l) t += gmat[(size_t)i * nobs + st + l] * Si[(size_t)j * n + l];
                gts[(size_t)(st + j) * D + i] = (1.0 / sigma_sar2) * t;
            }
        off += (size_t)n * n;
    }
    for (int io = s->nsar_total; io < nobs; ++io)
        sdvec[io] = s->dvec[io] / (sigma_gnss2 * pow(s->obs_sigma[io], 2));
    for (int i = 0; i < D; ++i) {
        double t = 0.0;
        for (int io = 0; io < nobs; ++io) t = t + gmat[(size_t)i * nobs + io] * sdvec[io];
        gsdvec[i] = t;
    }
    double dd = 0.0;
    for (int io = 0; io < nobs; ++io) dd = dd + s->dvec[io] * sdvec[io];
    *dsd = dd;
    for (int io = s->nsar_total; io < nobs; ++io)
        for (int i = 0; i < D; ++i)
            gts[(size_t)io * D + i] = gmat[(size_t)i * nobs + io] / (pow(s->obs_sigma[io], 2) * sigma_gnss2);
    for (int j = 0; j < D; ++j) {          // dgemm('n','n'): gsg = gts * G
        double *c = gsgmat + (size_t)j * D;
        for (int i = 0; i < D; ++i) c[i] = 0.0;
        for (int l = 0; l < nobs; ++l) {
            double t = gmat[(size_t)j * nobs + l];
            for (int i = 0; i < D; ++i) c[i] += t * gts[(size_t)l * D + i];
        }
    }
}

// ---------------------------------------------------------------------------
// Inner tempered SMC over slip (smc_slip.f90)
// ---------------------------------------------------------------------------
struct Inner {
    int D, N, nrow;
    const double *A, *b, *LL;
    double dsd;
    const int *lidx, *ltidx;
    const double *lval, *ltval;
    std::vector<double> alpha2;  // nrow (alpha2_full)
    double max_slip, lsar, lgnss;
    int nsar_total, ngnss, ntau, tf, max_stages;
    double cv;
    uint64_t seed, stream;
    int status;
};

static double cdf_norm(double x, double mu, double s2) { return (1.0 + erf((x - mu) / sqrt(2.0 * s2))) / 2.0; }
static double pdf_norm(double x, double mu, double s2) {
    double pi = 2.0 * asin(1.0);
    return exp(-((x - mu) * (x - mu)) / (2.0 * s2)) / sqrt(2.0 * pi * s2);
}

// slip_calc_likelihood (smc_slip.f90:56-104)
static double likelihood(const Inner &in, const double *sv) {
    int D = in.D;
    double v = 0.0;
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < i; ++j) v = v + sv[i] * in.A[(size_t)i * D + j] * sv[j];
    v = v * 2.0;
    for (int i = 0; i < D; ++i) v = v + sv[i] * in.A[(size_t)i * D + i] * sv[i];
    double dot = 0.0;
    for (int i = 0; i < D; ++i) dot = dot + in.b[i] * sv[i];
    return (v - 2.0 * dot + in.dsd) / 2.0 + in.nsar_total * in.lsar / 2.0 + 3.0 * in.ngnss * in.lgnss / 2.0;
}

// slip_calc_prior (smc_slip.f90:106-137)
static double prior(const Inner &in, const double *sv) {
    double p = 0.0;
    for (int i = 0; i < in.nrow; ++i) {
        double t = 0.0;
        for (int j = 0; j < 9; ++j) t = t + in.lval[9 * i + j] * sv[in.lidx[9 * i + j]];
        p = p + t * t / (2.0 * in.alpha2[i]);
    }
    return p;
}

// slip_calc_grad (smc_slip.f90:139-182)
static void gradient(const Inner &in, const double *sv, double gamma, double *grad, double *ls) {
    int D = in.D;
    for (int i = 0; i < D; ++i) grad[i] = 0.0;
    for (int j = 0; j < D; ++j) {
        double t = sv[j];
        for (int i = 0; i < D; ++i) grad[i] += t * in.A[(size_t)j * D + i];
    }
    for (int i = 0; i < D; ++i) { grad[i] = grad[i] - in.b[i]; grad[i] = grad[i] * gamma; }
    for (int r = 0; r < in.nrow; ++r) {
        double t = 0.0;
        for (int j = 0; j < 9; ++j) t = t + in.lval[9 * r + j] * sv[in.lidx[9 * r + j]];
        ls[r] = t / in.alpha2[r];
    }
    for (int i = 0; i < D; ++i) {
        double t = 0.0;
        for (int j = 0; j < 9; ++j) t = t + in.ltval[9 * i + j] * ls[in.ltidx[9 * i + j]];
        grad[i] = grad[i] + t;
    }
}

// reflection loop (smc_slip.f90:787-799); mod(idim,1)==0 always selects the
// [0, max_slip] branch.
static inline void reflect(double &x, double &p, double mx, int &status) {
    long it = 0;
    while (x < 0.0 || x > mx) {
        if (x > mx) { x = 2.0 * mx - x; p = -p; }
        if (x < 0.0) { x = -x; p = -p; }
        if (++it > 1000000) { status |= ORC_ST_REFLECT_CAP; break; }
    }
}

// slip_leapfrog (smc_slip.f90:732-917)
static void leapfrog(Inner &in, double &ham_cur, double post_cur, double *p, const double *cov,
                     double *cand, double dtau, int ntau, double gamma, const double *cur,
                     double &L_c, double &P_c, double &post_c, double &ham_c,
                     std::vector<double> &grad, std::vector<double> &ls) {
    int D = in.D;
    ham_cur = post_cur;
    for (int i = 0; i < D; ++i) ham_cur = ham_cur + p[i] * cov[i] * p[i] / 2.0;
    gradient(in, cand, gamma, grad.data(), ls.data());
    for (int i = 0; i < D; ++i) p[i] = p[i] - grad[i] * 5e-1 * dtau;
    for (int it = 0; it < ntau; ++it) {
        for (int i = 0; i < D; ++i) {
            cand[i] = cand[i] + cov[i] * p[i] * dtau;
            if (fabs(cand[i]) > 1e3) {
                for (int k = 0; k < D; ++k) cand[k] = cur[k];
                ham_c = 1e20;
                return;
            }
            reflect(cand[i], p[i], in.max_slip, in.status);
        }
        gradient(in, cand, gamma, grad.data(), ls.data());
        for (int i = 0; i < D; ++i) p[i] = p[i] - grad[i] * dtau;
    }
    for (int i = 0; i < D; ++i) {
        cand[i] = cand[i] + cov[i] * p[i] * 5e-1 * dtau;
        if (fabs(cand[i]) > 1e3) {
            for (int k = 0; k < D; ++k) cand[k] = cur[k];
            ham_c = 1e20;
            return;
        }
        reflect(cand[i], p[i], in.max_slip, in.status);
    }
    L_c = likelihood(in, cand);
    P_c = prior(in, cand);
    post_c = gamma * L_c + P_c;
    ham_c = post_c;
    for (int i = 0; i < D; ++i) ham_c = ham_c + p[i] * cov[i] * p[i] / 2.0;
}

// binary128 residual-systematic resampling (smc_slip.f90:572-589,
// smc_fault.f90:572-590)
static void resample_q(const double *w, int n, int count_n, quad u, int32_t *a) {
    quad dn = (quad)count_n;
    u = u / dn;
    for (int i = 0; i < n; ++i) {
        a[i] = (int32_t)q_floor(((quad)w[i] - u) * dn) + 1;
        u = u + (quad)a[i] / dn - (quad)w[i];
    }
}

extern "C" void orc_resample(const double *w, int32_t n, double u_hi, double u_lo, int32_t *counts) {
    resample_q(w, n, n, (quad)u_hi + (quad)u_lo, counts);
}

// sort.cpp:3-7 — index[] (1-based) ordered by arr[index-1] descending with
// the non-stable std::sort.
extern "C" void orc_qsort_(int32_t *arr, int32_t *index, int32_t *n) {
    std::sort(index, index + (*n), [&](int32_t a, int32_t b) { return arr[a - 1] > arr[b - 1]; });
}

static quad quad_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage) {
    double h, l;
    orc_quad_uniform(seed, stream, purpose, stage, &h, &l);
    return (quad)h + (quad)l;
}

// slip_smc_exec (smc_slip.f90:1445-1663) after the Gram precompute
static double inner_smc(Inner &in, double *particles, double *Ls, double *Ps, orc_inner_trace *trace) {
    int D = in.D, N = in.N;
    std::vector<double> cur(D), cand(D), p(D), grad(D), ls(in.nrow), w(N), mean(D), cov(D);
    std::vector<double> pnew((size_t)N * D), Lnew(N), Pnew(N), dtau_ls(N, exp(-5.0));
    std::vector<int32_t> assigned(N), id_start(N);
    double log_dtau_upper = 0.0, log_dtau_lower = -1e1;

    // slip_gen_init_particles (smc_slip.f90:184-287)
    for (int i = 0; i < D; ++i) cur[i] = 0.0;
    for (int k = 0; k < N; ++k) {
        for (int i = 0; i < D; ++i) {
            double s2 = pow(in.LL[(size_t)i * D + i] / in.alpha2[i], -1.0);
            double mu = 0.0;
            for (int j = 0; j < i; ++j) mu = mu - in.LL[(size_t)j * D + i] / in.alpha2[i] * cur[j] * s2;
            for (int j = i + 1; j < D; ++j) mu = mu - in.LL[(size_t)j * D + i] / in.alpha2[i] * cur[j] * s2;
            double v1 = orc_normal(in.seed, in.stream, RNG_GIBBS, 0, k, i);
            double x = mu + v1 * sqrt(s2);
            double fx = cdf_norm(x, mu, s2), f1 = cdf_norm(in.max_slip, mu, s2), f0 = cdf_norm(0.0, mu, s2);
            double y = mu, err = 1.0, yp = y + err;
            int cnt = 0;
            while (err > 1e-8 && cnt < 100) {
                y = y - (cdf_norm(y, mu, s2) - ((f1 - f0) * fx + f0)) / pdf_norm(y, mu, s2);
                err = fabs(y - yp);
                yp = y;
                cnt = cnt + 1;
            }
            if (cnt >= 100) in.status |= ORC_ST_NEWTON_CAP;
            cur[i] = y;
        }
        for (int i = 0; i < D; ++i) particles[(size_t)k * D + i] = cur[i];
    }
    for (int k = 0; k < N; ++k) {
        Ls[k] = likelihood(in, particles + (size_t)k * D);
        Ps[k] = prior(in, particles + (size_t)k * D);
    }

    int iter = 1;
    double gamma = 0.0, neglog = 0.0;
    if (trace) trace->nstage = 0;
    while (1.0 - gamma > 10e-8) {
        // slip_find_next_gamma (smc_slip.f90:314-387)
        double gprev = gamma, minL = Ls[0];
        for (int k = 0; k < N; ++k) minL = std::min(minL, Ls[k]);
        double lower = gprev, upper = 1.0, err = 1.0, g = 1.0, dg;
        long cnt = 0;
        while (err > 1e-10) {
            g = (lower + upper) / 2.0;
            dg = g - gprev;
            for (int k = 0; k < N; ++k) w[k] = exp(-dg * (Ls[k] - minL));
            double m = 0.0;
            for (int k = 0; k < N; ++k) m = m + w[k];
            m = m / N;
            double sd = 0.0;
            for (int k = 0; k < N; ++k) sd = sd + (w[k] - m) * (w[k] - m);
            sd = sd / N;
            sd = sqrt(sd);
            double cv = sd / m;
            if (cv > in.cv) upper = g; else lower = g;
            err = fabs(cv - in.cv);
            if (fabs(g - 1.0) < 1e-10) break;
            if (++cnt > 100000) { in.status |= ORC_ST_BISECT_CAP; break; }
        }
        double ev = 0.0;
        dg = g - gprev;
        for (int k = 0; k < N; ++k) ev = ev + exp(-dg * (Ls[k] - minL));
        ev = ev / N;
        double inc = -log(ev) + dg * minL;
        gamma = g;
        neglog = neglog + inc;
        if (trace) { trace->gamma[trace->nstage] = gamma; trace->neglog_inc[trace->nstage] = inc; }
        if (iter > in.max_stages) {
            neglog = 1e10;
            in.status |= ORC_ST_STAGE_CAP;
            if (trace) trace->nstage++;
            break;
        }
        // slip_normalize_weights (:465-483)
        quad sum = 0;
        for (int k = 0; k < N; ++k) sum = sum + (quad)w[k];
        for (int k = 0; k < N; ++k) w[k] = (double)((quad)w[k] / sum);
        // slip_calc_mean_particles (:485-505), slip_calc_cov_particles (:507-570)
        {
            std::vector<quad> md(D, (quad)0), cd(D, (quad)0);
            for (int k = 0; k < N; ++k) {
                double wt = w[k];
                for (int i = 0; i < D; ++i) md[i] = md[i] + (quad)(wt * particles[(size_t)k * D + i]);
            }
            for (int i = 0; i < D; ++i) mean[i] = (double)md[i];
            for (int k = 0; k < N; ++k) {
                double wt = w[k];
                for (int i = 0; i < D; ++i) {
                    double di = particles[(size_t)k * D + i] - mean[i];
                    cd[i] = cd[i] + (quad)(wt * di * di);
                }
            }
            for (int i = 0; i < D; ++i) {
                cov[i] = (double)cd[i];
                if (fabs(cov[i]) < 1e-3) cov[i] = 1e-3;
            }
        }
        // slip_resample_particles (:572-589)
        resample_q(w.data(), N, N, quad_uniform(in.seed, in.stream, RNG_RESAMPLE, iter), assigned.data());
        if (trace && trace->assigned)
            memcpy(trace->assigned + (size_t)trace->nstage * N, assigned.data(), N * sizeof(int32_t));
        if (trace) trace->nstage++;
        id_start[0] = 0;
        for (int k = 0; k < N - 1; ++k) id_start[k + 1] = id_start[k] + assigned[k];

        // slip_hmc_tuning (:919-1214)
        {
            int tcnt = 0;
            for (int k = 0; k < N; k += in.tf)
                for (int j = id_start[k]; j < id_start[k] + assigned[k]; ++j) {
                    ++tcnt;
                    double ld = orc_uniform(in.seed, in.stream, RNG_TUNE_DTAU, iter, j, 0);
                    ld = log_dtau_lower + ld * (log_dtau_upper - log_dtau_lower);
                    dtau_ls[j] = exp(ld);
                }
            if (tcnt > 0) {
                std::vector<double> score(N, -1.0), wh(N, -1.0), dnew(N);
                std::vector<int32_t> nh(N, 0);
                for (int k = 0; k < N; k += in.tf) {
                    for (int i = 0; i < D; ++i) cur[i] = particles[(size_t)k * D + i];
                    double Lc = Ls[k], Pc = Ps[k], post = gamma * Lc + Pc;
                    for (int j = id_start[k]; j < id_start[k] + assigned[k]; ++j) {
                        double dtau = dtau_ls[j];
                        for (int i = 0; i < D; ++i) cand[i] = cur[i];
                        for (int i = 0; i < D; ++i)
                            p[i] = orc_normal(in.seed, in.stream, RNG_TUNE_MOM, iter, j, i) / sqrt(cov[i]);
                        double hc = 0, Lx = 0, Px = 0, postx = 0, hx = 0;
                        leapfrog(in, hc, post, p.data(), cov.data(), cand.data(), dtau, in.ntau, gamma,
                                 cur.data(), Lx, Px, postx, hx, grad, ls);
                        double dham = hc - hx, sc = 0.0;
                        for (int i = 0; i < D; ++i) sc = sc + ((cand[i] - cur[i]) * (cand[i] - cur[i])) / cov[i];
                        sc = sc * exp(std::min(0.0, dham));
                        score[j] = sc;
                        double mh = orc_uniform(in.seed, in.stream, RNG_TUNE_MH, iter, j, 0);
                        if (hc - hx > log(mh)) {
                            for (int i = 0; i < D; ++i) cur[i] = cand[i];
                            Lc = Lx; Pc = Px; post = postx;
                        }
                    }
                }
                double ssum = 0.0;
                for (int k = 0; k < N; k += in.tf)
                    for (int j = id_start[k]; j < id_start[k] + assigned[k]; ++j) ssum = ssum + score[j];
                if (ssum < 1e-5) {
                    ssum = 0.0;
                    for (int k = 0; k < N; k += in.tf)
                        for (int j = id_start[k]; j < id_start[k] + assigned[k]; ++j) { score[j] = 1.0; ssum = ssum + 1.0; }
                }
                std::vector<double> wsub;
                std::vector<int> jsub;
                for (int k = 0; k < N; k += in.tf)
                    for (int j = id_start[k]; j < id_start[k] + assigned[k]; ++j) {
                        wh[j] = score[j] / ssum;
                        wsub.push_back(wh[j]);
                        jsub.push_back(j);
                    }
                std::vector<int32_t> asub(wsub.size());
                resample_q(wsub.data(), (int)wsub.size(), N, quad_uniform(in.seed, in.stream, RNG_TUNE_RES, iter), asub.data());
                long tot = 0;
                for (size_t q = 0; q < asub.size(); ++q) tot += asub[q];
                if (tot != N) {
                    in.status |= ORC_ST_TUNE_COUNT;
                } else {
                    int c = 0;
                    for (size_t q = 0; q < asub.size(); ++q)
                        for (int r = 0; r < asub[q]; ++r) dnew[c++] = dtau_ls[jsub[q]];
                    for (int k = 0; k < N; ++k) dtau_ls[k] = dnew[k];
                }
                quad dm = 0;
                for (int k = 0; k < N; ++k) dm = dm + (quad)dtau_ls[k];
                dm = dm / (quad)N;
                log_dtau_upper = (double)(q_log(dm) + (quad)log(5.0));
                log_dtau_lower = (double)(q_log(dm) - (quad)log(5.0));
            }
        }
        // slip_hmc_sampling (:591-730)
        for (int k = 0; k < N; ++k) {
            for (int i = 0; i < D; ++i) cur[i] = particles[(size_t)k * D + i];
            double Lc = Ls[k], Pc = Ps[k], post = gamma * Lc + Pc;
            for (int j = id_start[k]; j < id_start[k] + assigned[k]; ++j) {
                double dtau = dtau_ls[j];
                for (int i = 0; i < D; ++i) cand[i] = cur[i];
                for (int i = 0; i < D; ++i) p[i] = orc_normal(in.seed, in.stream, RNG_SMP_MOM, iter, j, i) / sqrt(cov[i]);
                double hc = 0, Lx = 0, Px = 0, postx = 0, hx = 0;
                leapfrog(in, hc, post, p.data(), cov.data(), cand.data(), dtau, in.ntau, gamma, cur.data(),
                         Lx, Px, postx, hx, grad, ls);
                double mh = orc_uniform(in.seed, in.stream, RNG_SMP_MH, iter, j, 0);
                if (hc - hx > log(mh)) {
                    for (int i = 0; i < D; ++i) cur[i] = cand[i];
                    Lc = Lx; Pc = Px; post = postx;
                }
                for (int i = 0; i < D; ++i) pnew[(size_t)j * D + i] = cur[i];
                Lnew[j] = Lc; Pnew[j] = Pc;
            }
        }
        memcpy(particles, pnew.data(), (size_t)N * D * sizeof(double));
        memcpy(Ls, Lnew.data(), N * sizeof(double));
        memcpy(Ps, Pnew.data(), N * sizeof(double));
        iter = iter + 1;
    }
    if (!std::isfinite(neglog)) in.status |= ORC_ST_NONFINITE;
    return neglog;
}

// fault_calc_likelihood (smc_fault.f90:66-292)
extern "C" int orc_fault_likelihood(const orc_setup *s, const double *theta, uint64_t seed, uint64_t stream,
                                    double *neglog, double *particles_out, double *likelihood_out,
                                    double *prior_out, orc_inner_trace *trace) {
    std::vector<Plane> pl;
    planes_of(s, theta, pl);
    Mesh m;
    discretize(s, pl, m);
    Lap lp;
    laplacian_impl(s, pl, m, lp);
    int D = m.D, nobs = s->nobs, N = s->nparticle_slip;
    std::vector<double> gmat((size_t)nobs * D);
    greens_impl(s, pl, m, gmat.data());
    double la2, lsar, lgnss;
    orc_hyper(s, theta, &la2, &lsar, &lgnss);
    std::vector<double> A((size_t)D * D), b(D);
    double dsd;
    orc_gram(s, gmat.data(), exp(lsar), exp(lgnss), A.data(), b.data(), &dsd);
    Inner in;
    in.D = D; in.N = N; in.nrow = lp.nrow;
    in.A = A.data(); in.b = b.data(); in.dsd = dsd; in.LL = lp.ll.data();
    in.lidx = lp.lidx.data(); in.lval = lp.lval.data(); in.ltidx = lp.ltidx.data(); in.ltval = lp.ltval.data();
    in.alpha2.assign(lp.nrow, exp(la2));
    in.max_slip = s->max_slip; in.lsar = lsar; in.lgnss = lgnss;
    in.nsar_total = s->nsar_total; in.ngnss = s->ngnss;
    in.ntau = s->ntau; in.tf = s->tuning_factor; in.max_stages = s->max_stages; in.cv = s->cv_inner;
    in.seed = seed; in.stream = stream; in.status = 0;
    std::vector<double> parts((size_t)N * D), Ls(N), Ps(N);
    *neglog = inner_smc(in, parts.data(), Ls.data(), Ps.data(), trace);
    if (particles_out) memcpy(particles_out, parts.data(), parts.size() * sizeof(double));
    if (likelihood_out) memcpy(likelihood_out, Ls.data(), N * sizeof(double));
    if (prior_out) memcpy(prior_out, Ps.data(), N * sizeof(double));
    return in.status;
}

// The inner target's pieces at one slip vector x for geometry theta: the
// likelihood (slip_calc_likelihood, smc_slip.f90:56-104), the prior
// (slip_calc_prior, :106-137) and the tempered gradient gamma * dL/dx + dP/dx
// (slip_calc_grad, :139-182), on the same G, Gram products and Laplacian as
// orc_fault_likelihood.  For the finite-difference check of the gradient.
extern "C" int orc_slip_energy(const orc_setup *s, const double *theta, double gamma, const double *x,
                               double *lik, double *pri, double *grad) {
    std::vector<Plane> pl;
    planes_of(s, theta, pl);
    Mesh m;
    discretize(s, pl, m);
    Lap lp;
    laplacian_impl(s, pl, m, lp);
    int D = m.D, nobs = s->nobs;
    std::vector<double> gmat((size_t)nobs * D);
    greens_impl(s, pl, m, gmat.data());
    double la2, lsar, lgnss;
    orc_hyper(s, theta, &la2, &lsar, &lgnss);
    std::vector<double> A((size_t)D * D), b(D);
    double dsd;
    orc_gram(s, gmat.data(), exp(lsar), exp(lgnss), A.data(), b.data(), &dsd);
    Inner in;
    in.D = D; in.N = 1; in.nrow = lp.nrow;
    in.A = A.data(); in.b = b.data(); in.dsd = dsd; in.LL = lp.ll.data();
    in.lidx = lp.lidx.data(); in.lval = lp.lval.data(); in.ltidx = lp.ltidx.data(); in.ltval = lp.ltval.data();
    in.alpha2.assign(lp.nrow, exp(la2));
    in.lsar = lsar; in.lgnss = lgnss; in.nsar_total = s->nsar_total; in.ngnss = s->ngnss;
    std::vector<double> ls(lp.nrow);
    *lik = likelihood(in, x);
    *pri = prior(in, x);
    gradient(in, x, gamma, grad, ls.data());
    return D;
}

extern "C" int orc_fault_likelihood_batch(const orc_setup *s, int32_t n, const double *theta, uint64_t seed,
                                          const uint64_t *streams, double *neglog, int32_t *status,
                                          int32_t nthreads) {
    int nd = ndim_fault_of(s);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int t = 0; t < n; ++t) {
        int st = orc_fault_likelihood(s, theta + (size_t)t * nd, seed, streams[t], &neglog[t], nullptr,
                                      nullptr, nullptr, nullptr);
        if (status) status[t] = st;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Outer SMC over geometry, fault_smc_exec (smc_fault.f90:785-1075), uniform
// prior box (gsmc = .false.).
// ---------------------------------------------------------------------------
static int cholesky_lower(double *a, int n) {   // dpotrf('L'), column-major
    for (int j = 0; j < n; ++j) {
        double d = a[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= a[(size_t)k * n + j] * a[(size_t)k * n + j];
        if (!(d > 0.0)) return j + 1;
        d = sqrt(d);
        a[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double v = a[(size_t)j * n + i];
            for (int k = 0; k < j; ++k) v -= a[(size_t)k * n + i] * a[(size_t)k * n + j];
            a[(size_t)j * n + i] = v / d;
        }
    }
    return 0;
}

// dtrmv('l','n','n'): z := L z with L lower-triangular, column-major (the
// reference BLAS column order)
static void trmv_lower(const double *L, int nd, double *z) {
    for (int jj = nd - 1; jj >= 0; --jj) {
        double t = z[jj];
        for (int ii = nd - 1; ii > jj; --ii) z[ii] += t * L[(size_t)jj * nd + ii];
        z[jj] *= L[(size_t)jj * nd + jj];
    }
}

// fault_calc_neglog_q (smc_fault.f90:9-27): -log N(x; qmean, qcov)
static double neglog_q(const orc_gsmc *q, const double *x, int nd) {
    double pi = 2.0 * asin(1.0);
    std::vector<double> delta(nd);
    for (int d = 0; d < nd; ++d) delta[d] = x[d] - q->qmean[d];
    double tmp = 0.0;
    for (int j = 0; j < nd; ++j)
        for (int i = 0; i < nd; ++i) tmp = tmp + delta[i] * q->qcov_inv[(size_t)j * nd + i] * delta[j];
    return tmp / 2.0 + log(2.0 * pi) * nd / 2.0 + q->log_qcov_det / 2.0;
}

extern "C" int orc_fault_smc(const orc_setup *s, const double *range, int32_t N, int32_t numprocs,
                             uint64_t seed, int32_t nthreads, double *particles_out, double *likelihood_out,
                             double *evidence_out, int32_t *nstage_out, double *gamma_out, const orc_gsmc *gq) {
    int nd = ndim_fault_of(s);
    std::vector<double> parts((size_t)N * nd), Ls(N), w(N), mean(nd), cov((size_t)nd * nd), qs(N, 0.0);
    std::vector<int32_t> assigned(N), sorted(N);
    int status = 0;
    // fault_sample_init_particles (smc_fault.f90:29-64)
    if (gq) {
        std::vector<double> z(nd);
        for (int i = 0; i < N; ++i) {
            for (int d = 0; d < nd; ++d) z[d] = orc_normal(seed, OUTER_STREAM, RNG_OUT_QINIT, 0, i, d);
            trmv_lower(gq->qcov_chol, nd, z.data());
            for (int d = 0; d < nd; ++d) parts[(size_t)i * nd + d] = z[d] + gq->qmean[d];
        }
    } else {
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < nd; ++d) {
                double u = orc_uniform(seed, OUTER_STREAM, RNG_OUT_INIT, 0, i, d);
                parts[(size_t)i * nd + d] = range[2 * d] + u * (range[2 * d + 1] - range[2 * d]);
            }
    }
    {
        std::vector<uint64_t> st(N);
        std::vector<int32_t> stv(N);
        for (int i = 0; i < N; ++i) st[i] = eval_stream(0, 0, i);
        orc_fault_likelihood_batch(s, N, parts.data(), seed, st.data(), Ls.data(), stv.data(), nthreads);
        for (int i = 0; i < N; ++i) status |= stv[i];
        // work_eval_init_particles (smc_fault.f90:350-353)
        if (gq)
            for (int i = 0; i < N; ++i) qs[i] = neglog_q(gq, &parts[(size_t)i * nd], nd);
    }
    double gamma = 0.0, evidence = 0.0;
    int iter = 1;
    while (1.0 - gamma > pow(10.0, -8.0)) {
        if (s->max_outer_stages != 0 && iter > std::max(s->max_outer_stages, 0)) break;
        // fault_find_next_gamma (:392-485); GSMC tempers L - q
        std::vector<double> nlr(N);
        for (int i = 0; i < N; ++i) nlr[i] = gq ? Ls[i] - qs[i] : Ls[i];
        double gprev = gamma, minL = nlr[0];
        for (int i = 0; i < N; ++i) minL = std::min(minL, nlr[i]);
        double lower = gprev, upper = 1.0, err = 1.0, dg;
        int cnt = 0;
        while (err > pow(10.0, -8.0)) {
            gamma = (lower + upper) / 2.0;
            dg = gamma - gprev;
            for (int i = 0; i < N; ++i) w[i] = exp(-dg * (nlr[i] - minL));
            double m = 0.0;
            for (int i = 0; i < N; ++i) m = m + w[i];
            m = m / N;
            double sd = 0.0;
            for (int i = 0; i < N; ++i) sd = sd + (w[i] - m) * (w[i] - m);
            sd = sqrt(sd / N);
            double cv = sd / m;
            if (cv > s->cv_outer) upper = gamma; else lower = gamma;
            err = fabs(cv - s->cv_outer);
            if (fabs(gamma - 1.0) < pow(10.0, -8.0)) break;
            if (cnt > 1000) break;
            cnt = cnt + 1;
        }
        double ev = 0.0;
        dg = gamma - gprev;
        for (int i = 0; i < N; ++i) ev = ev + exp(-dg * (nlr[i] - minL));
        ev = ev / N;
        evidence = evidence - log(ev) + dg * minL;
        if (gamma_out && iter <= 1024) gamma_out[iter - 1] = gamma;
        // fault_normalize_weights, fault_calc_mean_particles, fault_calc_cov_particles
        double sum = 0.0;
        for (int i = 0; i < N; ++i) sum = sum + w[i];
        for (int i = 0; i < N; ++i) w[i] = w[i] / sum;
        for (int d = 0; d < nd; ++d) mean[d] = 0.0;
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < nd; ++d) mean[d] = mean[d] + w[i] * parts[(size_t)i * nd + d];
        for (size_t q = 0; q < cov.size(); ++q) cov[q] = 0.0;
        for (int i = 0; i < N; ++i) {
            double wt = w[i];
            for (int jd = 0; jd < nd; ++jd)
                for (int id = jd; id < nd; ++id)
                    cov[(size_t)jd * nd + id] = cov[(size_t)jd * nd + id] +
                        wt * (parts[(size_t)i * nd + id] - mean[id]) * (parts[(size_t)i * nd + jd] - mean[jd]);
        }
        for (size_t q = 0; q < cov.size(); ++q) cov[q] = cov[q] * 0.04;
        if (cholesky_lower(cov.data(), nd) != 0) status |= ORC_ST_NONFINITE;
        // fault_resample_particles (quad)
        resample_q(w.data(), N, N, quad_uniform(seed, OUTER_STREAM, RNG_OUT_RES, iter), assigned.data());
        // fault_reorder_to_send (:592-637) with qsort_ (sort.cpp)
        {
            std::vector<int32_t> ta = assigned;
            std::vector<double> tp = parts, tl = Ls, tq = qs;
            for (int i = 0; i < N; ++i) sorted[i] = i + 1;
            int32_t nn = N;
            orc_qsort_(assigned.data(), sorted.data(), &nn);
            int ws = N / numprocs;
            for (int ip = 0; ip < numprocs; ++ip)
                for (int k = 0; k < ws; ++k) {
                    int org = sorted[k * numprocs + ip] - 1;
                    int nw = ip * ws + k;
                    assigned[nw] = ta[org];
                    for (int d = 0; d < nd; ++d) parts[(size_t)nw * nd + d] = tp[(size_t)org * nd + d];
                    Ls[nw] = tl[org];
                    qs[nw] = tq[org];
                }
        }
        // work_mcmc_sampling (:639-783): parents re-evaluated, then chained MH
        // children.  Evaluations are batched by chain position; every chain
        // still sees its own sequence of proposals.
        std::vector<int32_t> start(N);
        start[0] = 0;
        for (int i = 0; i < N - 1; ++i) start[i + 1] = start[i] + assigned[i];
        std::vector<double> curp = parts, Lcur(N), newp((size_t)N * nd), newL(N), qcur = qs, newq(N, 0.0);
        {
            std::vector<uint64_t> st(N);
            std::vector<int32_t> stv(N);
            for (int i = 0; i < N; ++i) st[i] = eval_stream(iter, 0, i);
            orc_fault_likelihood_batch(s, N, parts.data(), seed, st.data(), Lcur.data(), stv.data(), nthreads);
            for (int i = 0; i < N; ++i) status |= stv[i];
        }
        int maxa = 0;
        for (int i = 0; i < N; ++i) maxa = std::max(maxa, (int)assigned[i]);
        for (int r = 0; r < maxa; ++r) {
            std::vector<int> who;
            std::vector<double> cand;
            std::vector<uint64_t> st;
            for (int i = 0; i < N; ++i) {
                if (assigned[i] <= r) continue;
                int j = start[i] + r;
                std::vector<double> z(nd), x(nd);
                for (int d = 0; d < nd; ++d) z[d] = orc_normal(seed, OUTER_STREAM, RNG_OUT_PROP, iter, j, d);
                trmv_lower(cov.data(), nd, z.data());
                for (int d = 0; d < nd; ++d) x[d] = curp[(size_t)i * nd + d] + z[d];
                for (int d = 0; d < nd; ++d) {
                    double lo = range[2 * d], hi = range[2 * d + 1];
                    if (hi - lo > 1e-3) {
                        if (x[d] < lo) x[d] = std::min(2.0 * lo - x[d], hi);
                        if (x[d] > hi) x[d] = std::max(2.0 * hi - x[d], lo);
                    }
                }
                who.push_back(i);
                cand.insert(cand.end(), x.begin(), x.end());
                st.push_back(eval_stream(iter, 1, j));
            }
            int nb = (int)who.size();
            std::vector<double> Lc(nb);
            std::vector<int32_t> stv(nb);
            orc_fault_likelihood_batch(s, nb, cand.data(), seed, st.data(), Lc.data(), stv.data(), nthreads);
            for (int q = 0; q < nb; ++q) {
                status |= stv[q];
                int i = who[q], j = start[i] + r;
                double mh = orc_uniform(seed, OUTER_STREAM, RNG_OUT_MH, iter, j, 0);
                // work_mcmc_sampling's test (smc_fault.f90:748-771)
                double qc = gq ? neglog_q(gq, &cand[(size_t)q * nd], nd) : 0.0;
                double lhs = gq ? gamma * (Lcur[i] - Lc[q]) + (1.0 - gamma) * (qcur[i] - qc) : gamma * (Lcur[i] - Lc[q]);
                if (lhs > log(mh)) {
                    for (int d = 0; d < nd; ++d) curp[(size_t)i * nd + d] = cand[(size_t)q * nd + d];
                    Lcur[i] = Lc[q];
                    qcur[i] = qc;
                }
                newL[j] = Lcur[i];
                newq[j] = qcur[i];
                for (int d = 0; d < nd; ++d) newp[(size_t)j * nd + d] = curp[(size_t)i * nd + d];
            }
        }
        parts = newp;
        Ls = newL;
        qs = newq;
        iter = iter + 1;
        if (iter > 100000) break;
    }
    if (particles_out) memcpy(particles_out, parts.data(), parts.size() * sizeof(double));
    if (likelihood_out) memcpy(likelihood_out, Ls.data(), N * sizeof(double));
    *evidence_out = evidence;
    *nstage_out = iter - 1;
    return status;
}
