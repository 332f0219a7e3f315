// Shared device helpers: error plumbing, the Philox4x64-10 random stream and
// the per-theta geometry record.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/smcgpu.h"

#define SMC_HD __host__ __device__ __forceinline__

namespace smc {

// ---------------------------------------------------------------------------
// Random stream.  The reference draws from the Fortran intrinsic
// random_number with clipping at 1e-5 (random_number_correction,
// smc_slip.f90:8-24).  Here every draw is addressed by
// key = (seed, stream) and counter = (stage<<32 | purpose, i, j>>2, 0) of
// Philox4x64-10 (Salmon et al., SC'11); output word j&3 is used.  The stream
// equals numpy.random.Philox with the counter pre-incremented.
// ---------------------------------------------------------------------------
enum RngPurpose : uint32_t {
    RNG_GIBBS = 1, RNG_TUNE_DTAU = 2, RNG_TUNE_MOM = 3, RNG_TUNE_MH = 4, RNG_TUNE_RES = 5,
    RNG_SMP_MOM = 6, RNG_SMP_MH = 7, RNG_RESAMPLE = 8,
    RNG_OUT_INIT = 16, RNG_OUT_RES = 17, RNG_OUT_PROP = 18, RNG_OUT_MH = 19, RNG_OUT_QINIT = 20
};
static constexpr uint64_t OUTER_STREAM = ~0ull;

SMC_HD uint64_t eval_stream(uint32_t iter, uint32_t kind, uint64_t slot) {
    return ((uint64_t)iter << 40) | ((uint64_t)kind << 39) | slot;
}

SMC_HD void mulhilo64(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
#ifdef __CUDA_ARCH__
    hi = __umul64hi(a, b);
    lo = a * b;
#else
    unsigned __int128 p = (unsigned __int128)a * b;
    hi = (uint64_t)(p >> 64);
    lo = (uint64_t)p;
#endif
}

struct U64x4 { uint64_t v[4]; };

SMC_HD U64x4 philox4x64(uint64_t c0, uint64_t c1, uint64_t c2, uint64_t c3, uint64_t k0, uint64_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t hi0, lo0, hi1, lo1;
        mulhilo64(0xD2E7470EE14C6C93ull, c0, hi0, lo0);
        mulhilo64(0xCA5A826395121157ull, c2, hi1, lo1);
        uint64_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B97F4A7C15ull;
        k1 += 0xBB67AE8584CAA73Bull;
    }
    U64x4 o;
    o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
    return o;
}

SMC_HD uint64_t rng_raw(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, uint64_t i, uint64_t j) {
    U64x4 o = philox4x64(((uint64_t)stage << 32) | purpose, i, j >> 2, 0, seed, stream);
    return o.v[j & 3];
}

SMC_HD double clip_uniform(uint64_t raw) {
    double x = (double)(raw >> 11) * 0x1.0p-53;
    return x < 1e-5 ? 1e-5 : x;
}

SMC_HD double rng_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, uint64_t i, uint64_t j) {
    return clip_uniform(rng_raw(seed, stream, purpose, stage, i, j));
}

// Box-Muller sine branch (slip_BoxMuller, smc_slip.f90:26-38): one Philox
// block yields the (r, s) pairs of normals d = 2k and 2k+1.
__device__ __forceinline__ double rng_normal(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                                             uint64_t i, uint64_t d) {
    U64x4 o = philox4x64(((uint64_t)stage << 32) | purpose, i, d >> 1, 0, seed, stream);
    int b = (int)(d & 1) * 2;
    double r = clip_uniform(o.v[b]), s = clip_uniform(o.v[b + 1]);
    const double pi = 3.141592653589793;
    return sqrt(-2.0 * log(r)) * sin(2.0 * pi * s);
}

// FP32 uniform from the top 23 bits of a raw word, clipped like
// random_number_correction: integer and FP32 operations only
__device__ __forceinline__ float clip_uniform_f(uint64_t raw) {
    const float u = __uint_as_float(0x3F800000u | (uint32_t)(raw >> 41)) - 1.0f;
    return u < 1e-5f ? 1e-5f : u;
}

// MIXED normals: the same Philox blocks as rng_normal, FP32 arithmetic
__device__ __forceinline__ float rng_normal_f(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                                              uint64_t i, uint64_t d) {
    U64x4 o = philox4x64(((uint64_t)stage << 32) | purpose, i, d >> 1, 0, seed, stream);
    int b = (int)(d & 1) * 2;
    float r = clip_uniform_f(o.v[b]), s = clip_uniform_f(o.v[b + 1]);
    return sqrtf(-2.0f * __logf(r)) * __sinf(6.2831853f * s);
}
// both normals of one block: dimensions 2k and 2k+1
__device__ __forceinline__ float2 rng_normal2_f(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage,
                                                uint64_t i, uint64_t k) {
    U64x4 o = philox4x64(((uint64_t)stage << 32) | purpose, i, k, 0, seed, stream);
    const float r0 = clip_uniform_f(o.v[0]), s0 = clip_uniform_f(o.v[1]);
    const float r1 = clip_uniform_f(o.v[2]), s1 = clip_uniform_f(o.v[3]);
    return make_float2(sqrtf(-2.0f * __logf(r0)) * __sinf(6.2831853f * s0),
                       sqrtf(-2.0f * __logf(r1)) * __sinf(6.2831853f * s1));
}

// exact FP32 value of a double that holds an FP32 number (MIXED particle
// values), by integer operations; other values fall back to a conversion
__device__ __forceinline__ float f32_of_f32valued(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const uint32_t hi = (uint32_t)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7FF);
    if (e >= 897 && e <= 1150 && (b & 0x1FFFFFFFull) == 0)
        return __uint_as_float((hi & 0x80000000u) | ((uint32_t)(e - 896) << 23) | (uint32_t)((b >> 29) & 0x7FFFFF));
    return (b << 1) == 0 ? __uint_as_float(hi & 0x80000000u) : (float)v;
}

// random_number_correction_dd: binary128 uniform carried as an exact 106-bit
// double-double.
SMC_HD void rng_quad_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, double &hi, double &lo) {
    U64x4 o = philox4x64(((uint64_t)stage << 32) | purpose, 0, 0, 0, seed, stream);
    hi = (double)(o.v[0] >> 11) * 0x1.0p-53;
    lo = (double)(o.v[1] >> 11) * 0x1.0p-106;
    // exact test of hi + lo < 1e-5: hi is a multiple of 2^-53 and lo < 2^-53,
    // and 1e-5 - hi is exact whenever it is below 2^-53 (Sterbenz).
    const double v = 1e-5;
    if (hi < v && (v - hi > 0x1.0p-53 || lo < v - hi)) { hi = v; lo = 0.0; }
}

// ---------------------------------------------------------------------------
// Per-theta plane record produced by the setup kernel.
// ---------------------------------------------------------------------------
struct PlaneGeom {
    double xf, yf, zf;          // fault centre (gfunc.f90:294-296)
    double strike, dip;         // degrees
    double lxi, leta;           // plane length / width
    double sin_s, cos_s;        // strike_rad = strike/180*pi (gfunc.f90:120, :77)
    double cos_dip, sin_dip;    // dip_rad = dip/180*pi (gfunc.f90:119)
    double sd, cd;              // DCCON0 (DC3Dfortran.f90:1236-1263)
    double dxi, deta;
};

}  // namespace smc
