// Residual-systematic resampling counts as a prefix scan.
//
// The reference runs the recurrence (smc_slip.f90:572-589)
//     u = u0/N;  a_i = floor((w_i - u) N) + 1;  u = u + a_i/N - w_i
// in binary128.  In exact arithmetic its partial sums telescope to
//     C_i = a_1 + ... + a_i = floor(N W_i - u0) + 1,   W_i = w_1 + ... + w_i,
// so the counts are differences of a floor of a prefix sum.  The device
// evaluates N W_i - u0 in double-double (error < 1e-25 for N <= 2^20); the
// binary128 recurrence accumulates at most ~N 2^-112 of rounding, so both
// agree whenever the fractional part of N W_i - u0 is farther than 1e-20 from
// an integer.  Closer cases are detected and recomputed by the serial
// binary128 recurrence on the device (q128.cuh), so the counts equal the
// reference's bit for bit.
#include "common.cuh"
#include "ddreal.cuh"
#include "kernels.h"
#include "q128.cuh"

namespace smc {

// Serial binary128 recurrence on one thread (the near-tie path).
__device__ void resample_q128_serial(const double *w, int n, int count_n, double u_hi, double u_lo, int *counts) {
    q128 dn = q128_from_int(count_n);
    q128 u = q128_add(q128_from_double(u_hi), q128_from_double(u_lo));
    u = q128_div(u, dn);
    for (int i = 0; i < n; ++i) {
        q128 wi = q128_from_double(w[i]);
        q128 t = q128_mul(q128_sub(wi, u), dn);
        long long a = q128_floor(t) + 1;
        counts[i] = (int)a;
        u = q128_sub(q128_add(u, q128_div(q128_from_int(a), dn)), wi);
    }
}

__global__ void resample_counts_kernel(const double *__restrict__ w, int n, int count_n, double u_hi, double u_lo,
                                       int *__restrict__ counts, int *__restrict__ flag) {
    __shared__ dd scratch[32];
    __shared__ int s_tie;
    __shared__ long long s_prevC;
    if (threadIdx.x == 0) { s_tie = 0; s_prevC = 0; }
    __syncthreads();
    dd carry = {0.0, 0.0};
    const double dn = (double)count_n;
    const dd u0 = {u_hi, u_lo};
    for (int base = 0; base < n; base += blockDim.x) {
        int i = base + threadIdx.x;
        dd v = {i < n ? w[i] : 0.0, 0.0};
        dd tot;
        dd incl = block_scan_dd(v, scratch, tot);
        incl = dd_add(carry, incl);
        carry = dd_add(carry, tot);
        // C_i = floor(N W_i - u0) + 1
        dd x = dd_add(dd_mul_d(incl, dn), dd_neg(u0));
        double frac;
        long long C = dd_floor(x, frac) + 1;
        if (i < n && (frac < 1e-20 || frac > 1.0 - 1e-20)) s_tie = 1;
        // previous C from the neighbouring lane / tile
        long long Cprev = __shfl_up_sync(0xffffffffu, C, 1);
        __shared__ long long s_lastC[32];
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 31) s_lastC[wid] = C;
        __syncthreads();
        if (lane == 0) Cprev = (wid == 0) ? s_prevC : s_lastC[wid - 1];
        if (i < n) counts[i] = (int)(C - Cprev);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_prevC = C;
        __syncthreads();
    }
    if (s_tie) {
        if (threadIdx.x == 0) {
            resample_q128_serial(w, n, count_n, u_hi, u_lo, counts);
            if (flag) *flag = 1;
        }
    } else if (threadIdx.x == 0 && flag) {
        *flag = 0;
    }
}

cudaError_t launch_resample_counts(const double *w, int n, double u_hi, double u_lo, int *counts, int *flag,
                                   cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    resample_counts_kernel<<<1, 1024, 0, s>>>(w, n, n, u_hi, u_lo, counts, flag);
    return cudaGetLastError();
}

}  // namespace smc
