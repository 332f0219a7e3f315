// Double-double arithmetic (error-free transformations of Knuth / Dekker,
// Shewchuk) and the block-wide prefix scan used by the resampling kernels.
#pragma once
#include <cuda_runtime.h>

namespace smc {

struct dd { double hi, lo; };

__device__ __forceinline__ dd two_sum(double a, double b) {
    double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dd quick_two_sum(double a, double b) {
    double s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dd dd_add(dd x, dd y) {
    dd s = two_sum(x.hi, y.hi), t = two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_add_d(dd x, double y) {
    dd s = two_sum(x.hi, y);
    s.lo += x.lo;
    return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_mul_d(dd x, double y) {
    double p = x.hi * y, e = fma(x.hi, y, -p);
    e = fma(x.lo, y, e);
    return quick_two_sum(p, e);
}
__device__ __forceinline__ dd dd_neg(dd x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ dd dd_shfl_up(dd x, int delta) {
    return {__shfl_up_sync(0xffffffffu, x.hi, delta), __shfl_up_sync(0xffffffffu, x.lo, delta)};
}

// floor of a normalised double-double and its fractional part (double)
__device__ __forceinline__ long long dd_floor(dd x, double &frac) {
    double f = floor(x.hi);
    if (f == x.hi) {
        double g = floor(x.lo);
        frac = x.lo - g;
        return (long long)f + (long long)g;
    }
    frac = (x.hi - f) + x.lo;
    return (long long)f;
}

// Inclusive double-double prefix scan over one block (blockDim.x a multiple
// of 32, <= 1024).  `carry` is the running total from earlier tiles; the
// returned value includes it.  Uses scratch[32] in shared memory.
__device__ __forceinline__ dd block_scan_dd(dd v, dd *scratch, dd &tile_total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        dd n = dd_shfl_up(v, o);
        if (lane >= o) v = dd_add(n, v);
    }
    if (lane == 31) scratch[wid] = v;
    __syncthreads();
    if (wid == 0) {
        dd t = lane < nw ? scratch[lane] : dd{0.0, 0.0};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            dd n = dd_shfl_up(t, o);
            if (lane >= o) t = dd_add(n, t);
        }
        if (lane < nw) scratch[lane] = t;
    }
    __syncthreads();
    if (wid > 0) v = dd_add(scratch[wid - 1], v);
    tile_total = scratch[nw - 1];
    __syncthreads();
    return v;
}

}  // namespace smc
