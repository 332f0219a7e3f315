// Inner tempered SMC over slip (slip_smc_exec, smc_slip.f90:1445-1663):
// one GROUP of W warps per geometry particle, persistent over all stages.
//
// The HMC children of one parent form a Metropolis chain
// (smc_slip.f90:591-730: child k starts where child k-1 stopped), so an
// inner stage is a set of chains of uneven length.  A group runs chain slots
// in lock step and refills a slot from the group's parent queue (sorted by
// descending child count) when its chain ends.  A leapfrog step of all slots
// is the product grad = M x of the stage matrix M = gamma A + L^T L / alpha^2
// with the slot tile x, followed by the element-wise momentum / position
// update, the reflection into [0, max_slip] and the blow-up test.  Random
// draws are addressed by (stage, purpose, child index, dimension), so the
// slot schedule does not change results.
//
// Four step engines share the stage-level code (bisection, normalisation,
// moments, resampling counts, parent queue, step-size tuning):
//
//  * CUDA cores (FP64 up to D = 128; MIXED up to 192 on request): every warp
//    of a group owns C = 8 slots and runs its own FMA GEMM M x out of shared
//    memory (lane l owns rows (l%16)*RT.. and slots (l/16)*4..), so a step
//    needs no synchronisation beyond the warp.  W = 1..8 warps per geometry,
//    chosen from the batch size.
//
//  * Warp-level tensor-core MMA (MIXED default, D <= 256): M and the slots'
//    offsets from the stage mean are split into BF16 hi + lo and multiplied
//    with mma.sync m16n8k16 as lo*hi + hi*lo + hi*hi in three FP32 chains;
//    each warp owns (16-row, 8-slot) tiles of a 16-warp group (one geometry
//    per CTA), an 8-warp group (two per CTA) or, up to D = 64, a 4-warp group
//    of 16 slots (four per CTA, ENG_MMAQ: the Gram matrix of the end-point
//    energies then comes from global memory).  Up to D = 128 M sits in shared
//    memory (in registers for the stage when it is small); above, M is kept in
//    global memory in fragment order and every warp streams its rows through
//    a cp.async ring (Layout::AGL).
//
//  * tcgen05 (MIXED, D <= 128, on request): one warpgroup per geometry.  M
//    is split into BF16 hi + lo (stacked 128/DP times to fill the 128-row
//    MMA) and the slot tile's offsets likewise; thread 0 issues
//    hi*hi + hi*lo + lo*hi as tcgen05.mma (M = 128, N = 2048/DP slots, K = 16
//    per instruction) into a tensor-memory accumulator, and every thread
//    reads back its row (one dimension) for 16 slots with tcgen05.ld.
//
//  * Global matrix (both precisions, any D up to 1024; one geometry per CTA of
//    16 warps): M lives in global memory, column-major, and every step streams
//    it once for the group's 16 slots; each thread owns rows of M and streams
//    its own entries through a private cp.async ring (gl_gemm).
//
// The tensor-core gradient error is O(2^-16) relative; the Metropolis test
// is exact for any deterministic gradient, and the end-point energies keep
// their FP32 / FP64 form, so only the acceptance rate can move.
//
// FP64 (T = double) follows the reference's algebra in FP64.  MIXED
// (T = float) runs the leapfrog in FP32 (or the tensor cores) about the stage
// mean sbar with the constant part of the gradient and the end-point energies
// formed in FP64, and the tempering bisection in FP32 before one FP64 pass
// for the weights and the evidence increment.
// This header holds the kernel and launcher templates; each inner_*.cu unit
// instantiates one family of them (so that the units compile in parallel)
// and inner.cu dispatches between the families.
#pragma once
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "ddreal.cuh"
#include "inner.h"
#include "q128.cuh"
#include "tc.cuh"

namespace smc {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int CW = 8;    // chain slots per warp (CUDA-core engine)
constexpr int CTW = 4;   // slots per lane
constexpr int RGW = 16;  // row groups per warp
constexpr uint32_t WAIT_TRIES = 1u << 22;   // bounded mbarrier wait
// step engines; ENG_MMAQ is the warp-MMA engine with 16 chain slots per
// geometry and the FP32 Gram matrix of the end-point energies read from global
// memory (L2), so that four geometries of 4 warps share one SM (D <= 64)
enum : int { ENG_CC = 0, ENG_TC = 1, ENG_MMA = 2, ENG_GL = 3, ENG_MMAQ = 4 };
__host__ __device__ constexpr bool is_mma(int e) { return e == ENG_MMA || e == ENG_MMAQ; }

// ---- warp-level tensor-core MMA (BF16 in, FP32 accumulate), m16n8k16
__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(tc::smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t r[2], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(tc::smem_u32(p)));
}
__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

// ---- 16-byte asynchronous global -> shared copies (L2 only), in commit groups
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(NPEND) : "memory"); }

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ double wmin(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double hsum(double v) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ dd wsum_dd(dd v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dd n = {__shfl_xor_sync(FULL, v.hi, o), __shfl_xor_sync(FULL, v.lo, o)};
        v = dd_add(v, n);
    }
    return v;
}
__device__ __forceinline__ dd wscan_dd(dd v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        dd n = dd_shfl_up(v, o);
        if (lane >= o) v = dd_add(n, v);
    }
    return v;
}
__device__ __forceinline__ int wexscan(int v, int lane, int &total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += n;
    }
    total = __shfl_sync(FULL, x, 31);
    return x - v;
}
__device__ __forceinline__ double dd_div_into_w(double w, dd s) {
    double q = w / s.hi;
    double r = fma(-q, s.hi, w) - q * s.lo;
    return q + r / s.hi;
}
// Reflection into [0, max_slip] with momentum flips (smc_slip.f90:787-799).
// The loop body runs once as predicated selects (a no-op inside the box, so
// the result equals the reference's loop), and the loop proper only for the
// rare multiple reflection: no divergent branch on the common path.
template <typename T>
__device__ __forceinline__ void reflect_w(T &x, T &p, T mx, int &flag) {
    const bool h = x > mx;
    x = h ? T(2) * mx - x : x;
    p = h ? -p : p;
    const bool l = x < T(0);
    x = l ? -x : x;
    p = l ? -p : p;
    if (x < T(0) || x > mx) {
        int it = 1;
        while (x < T(0) || x > mx) {
            if (x > mx) { x = T(2) * mx - x; p = -p; }
            if (x < T(0)) { x = -x; p = -p; }
            if (++it > 1000000) { flag |= SMCGPU_ST_REFLECT_CAP; break; }
        }
    }
}
// Blow-up test (|x| > 1e3 freezes the chain and rejects it,
// smc_slip.f90:800-806) and reflection, branch-free unless either fires
template <typename T>
__device__ __forceinline__ bool blow_or_reflect(T &x, T &p, T mx, int &flag) {
    const bool blow = (x < T(0) ? -x : x) > T(1e3);   // |x| in T itself (no promotion)
    T xr = x, pr = p;
    reflect_w<T>(xr, pr, mx, flag);
    x = blow ? x : xr;
    p = blow ? p : pr;
    return blow;
}
// MIXED reflection in closed form: the reference's loop folds x into
// [0, max_slip] by successive reflections at 0 and max_slip (a triangle wave
// of period 2 max_slip) and flips p once per reflection.  For |x| well
// beyond max_slip (the tuning pass draws step sizes up to 1) the loop runs
// |x|/max_slip times; here the fold and the parity of the reflection count
// are computed directly.  Same map up to rounding; entries inside the box
// are unchanged.  imx = 1/max_slip.
__device__ __forceinline__ void reflect_fold(float &x, float &p, float mx, float imx) {
    const bool neg = x < 0.0f, out = neg || x > mx;
    const float u = (neg ? -x : x) * imx;
    const float k = fmaxf(ceilf(u) - 1.0f, 0.0f);   // reflections after the first one of a negative x
    const float fr = u - k;                          // in (0, 1]
    const int ki = (int)k;
    const float xf = (ki & 1) ? (1.0f - fr) * mx : fr * mx;
    const int flips = ki + (neg ? 1 : 0);
    x = out ? xf : x;
    p = (out && (flips & 1)) ? -p : p;
}

// Sum of 16 per-slot values over the 32 lanes of a warp: afterwards lane l
// holds the total of slot l >> 1 (in v[0]); 16 exchanges instead of 80.
__device__ __forceinline__ double wreduce16(double v[16], int lane) {
#pragma unroll
    for (int o = 16, n = 16; o >= 2; o >>= 1, n >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < n / 2; ++i) {
            double send = up ? v[i] : v[i + n / 2];
            double keep = up ? v[i + n / 2] : v[i];
            v[i] = keep + __shfl_xor_sync(FULL, send, o);
        }
    }
    return v[0] + __shfl_xor_sync(FULL, v[0], 1);
}

// Sum of NV per-slot values over the 32 lanes of a warp: afterwards lane l
// holds the total of value l / (32 / NV) (NV = 8 or 16).
template <int NV>
__device__ __forceinline__ double wreduce_n(double v[NV], int lane) {
#pragma unroll
    for (int o = 16, n = NV; n >= 2; o >>= 1, n >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < n / 2; ++i) {
            double send = up ? v[i] : v[i + n / 2];
            double keep = up ? v[i + n / 2] : v[i];
            v[i] = keep + __shfl_xor_sync(FULL, send, o);
        }
    }
    double t = v[0];
#pragma unroll
    for (int o = 16 / NV; o >= 1; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
    return t;
}

// 4- or 8-byte asynchronous global -> shared copy (through L1), in commit
// groups; src_bytes = 0 writes zeros and reads nothing
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(tc::smem_u32(dst)), "l"(src), "n"(BYTES),
                 "r"(src_bytes)
                 : "memory");
}
// (d0, d1) += a * (b0, b1) as one packed FP32x2 FMA: each lane is an FP32 fma,
// rounded as fmaf
__device__ __forceinline__ void ffma2(float &d0, float &d1, float a, float b0, float b1) {
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %2};\n\t"
        "mov.b64 pb, {%3, %4};\n\t"
        "mov.b64 pd, {%0, %1};\n\t"
        "fma.rn.f32x2 pd, pa, pb, pd;\n\t"
        "mov.b64 {%0, %1}, pd;\n\t}"
        : "+f"(d0), "+f"(d1)
        : "f"(a), "f"(b0), "f"(b1));
}

// Global-matrix step product: acc[i][s] = sum_k Mg[k][r_i] X[k][s0 + s] for the
// thread's rows r_i = row0 + i * RP (column-major Mg with leading dimension
// D; the matrix is rewritten every stage) and its SPT slots of the shared
// operand X (row stride S).  Each element of Mg is used by one thread only, so
// every thread streams its own R entries of the columns k + 1 .. k + P - 1
// through a private ring of P column slots in shared memory (ring[(slot R + i)
// * NTH + tid]) with cp.async while it multiplies column k: a column needs a
// cp.async.wait_group and no barrier, and P columns of every thread are in
// flight instead of one blocking load.  A ring slot is refilled only after the
// thread's own read of it fed its FMAs.  Results equal the plain loop's.
template <typename T, int R, int SPT, int RP, int S, int P, int NTH>
__device__ __forceinline__ void gl_gemm(const T *Mg, int D, const T *__restrict__ X, int row0, int s0,
                                        T *ring, int tid, T acc[R][SPT]) {
    // columns travel in groups of CG (four when the ring holds a multiple of
    // four columns, else pairs): one commit group and one wait per group
    constexpr int CG = P % 4 == 0 ? 4 : 2;
    static_assert(P % CG == 0, "the ring holds whole column groups");
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int q = 0; q < SPT; ++q) acc[i][q] = T(0);
    // the thread's rows; rows beyond D (and columns beyond D) are copied as
    // zeros (cp.async zero fill, nothing read) from a clamped in-bounds address,
    // so the product loop needs no per-entry select
    int rowc[R], bytes_r[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const bool live = row0 + i * RP < D;
        rowc[i] = live ? row0 + i * RP : D - 1;
        bytes_r[i] = live ? (int)sizeof(T) : 0;
    }
    T *my = ring + tid;
    // columns k .. k + CG - 1 into ring slots slot .. slot + CG - 1, one commit group
    auto issue_group = [&](int k, int slot) {
#pragma unroll
        for (int j = 0; j < CG; ++j) {
            const int kk = k + j;
            const bool col = kk < D;
            const T *src = Mg + (size_t)(col ? kk : D - 1) * D;
#pragma unroll
            for (int i = 0; i < R; ++i)
                cp_async_zfill<sizeof(T)>(my + ((slot + j) * R + i) * NTH, src + rowc[i], col ? bytes_r[i] : 0);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int kk = 0; kk < P; kk += CG) issue_group(kk, kk);
    int slot = 0;
    for (int k = 0; k < D; k += CG) {
        // groups committed: column groups 0 .. (k + P) / CG - 1; at most P / CG - 1
        // pending means the group of columns k .. k + CG - 1 has landed
        cp_async_wait<P / CG - 1>();
#pragma unroll
        for (int j = 0; j < CG; ++j) {
            T mv[R];
#pragma unroll
            for (int i = 0; i < R; ++i) mv[i] = my[((slot + j) * R + i) * NTH];
            // columns past D are zero-filled slots: their products add 0; the
            // operand rows past D exist (X has DP rows, a multiple of 256) and are zero
            const T *xk = X + (k + j) * S + s0;   // 16-byte aligned: S and s0 are multiples of 8
            if constexpr (sizeof(T) == 4) {
#pragma unroll
                for (int q = 0; q < SPT; q += 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(xk + q);
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        ffma2(acc[i][q], acc[i][q + 1], (float)mv[i], v.x, v.y);
                        ffma2(acc[i][q + 2], acc[i][q + 3], (float)mv[i], v.z, v.w);
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < SPT; q += 2) {
                    const double2 v = *reinterpret_cast<const double2 *>(xk + q);
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        acc[i][q] = fma((double)mv[i], v.x, (double)acc[i][q]);
                        acc[i][q + 1] = fma((double)mv[i], v.y, (double)acc[i][q + 1]);
                    }
                }
            }
        }
        issue_group(k + P, slot);   // the next group into the slots just consumed
        slot = slot + CG == P ? 0 : slot + CG;
    }
}

// Group of W warps (W*32 threads) synchronised by named barrier id+1.
struct Group {
    int id, W, wl, lane, gt, nt;
    double *scr;   // 2*W doubles of scratch (also W dd)
    __device__ __forceinline__ void sync() const {
        if (W == 1) {
            __syncwarp();
        } else {
            asm volatile("bar.sync %0, %1;" ::"r"(id + 1), "r"(nt) : "memory");
        }
    }
    __device__ double sum(double v) const {
        v = wsum(v);
        if (W == 1) return v;
        sync();
        if (lane == 0) scr[wl] = v;
        sync();
        return wsum(lane < W ? scr[lane] : 0.0);   // warp partials combined by a second shuffle tree
    }
    // FP32 sums of two values in one round of barriers
    __device__ void sum2f(float &u, float &v) const {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            u += __shfl_xor_sync(FULL, u, o);
            v += __shfl_xor_sync(FULL, v, o);
        }
        if (W == 1) return;
        float *fs = (float *)scr;
        sync();
        if (lane == 0) { fs[wl] = u; fs[W + wl] = v; }
        sync();
        u = lane < W ? fs[lane] : 0.0f;
        v = lane < W ? fs[W + lane] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            u += __shfl_xor_sync(FULL, u, o);
            v += __shfl_xor_sync(FULL, v, o);
        }
    }
    // two sums in one round of barriers
    __device__ void sum2(double &u, double &v) const {
        u = wsum(u);
        v = wsum(v);
        if (W == 1) return;
        sync();
        if (lane == 0) { scr[wl] = u; scr[W + wl] = v; }
        sync();
        u = wsum(lane < W ? scr[lane] : 0.0);
        v = wsum(lane < W ? scr[W + lane] : 0.0);
    }
    __device__ double min(double v) const {
        v = wmin(v);
        if (W == 1) return v;
        sync();
        if (lane == 0) scr[wl] = v;
        sync();
        return wmin(lane < W ? scr[lane] : 1e300);
    }
    __device__ dd sum_dd(dd v) const {
        v = wsum_dd(v);
        if (W == 1) return v;
        dd *s = (dd *)scr;
        sync();
        if (lane == 0) s[wl] = v;
        sync();
        return wsum_dd(lane < W ? s[lane] : dd{0.0, 0.0});
    }
};

// Residual-systematic counts (scan form with the binary128 near-tie
// fallback, resample.cu) computed by one warp; returns the total.
__device__ long long warp_counts(const double *w, int n, int count_n, double u_hi, double u_lo, int *cnt, int lane) {
    dd carry = {0.0, 0.0};
    long long prevC = 0;
    const dd u0 = {u_hi, u_lo};
    const double dn = (double)count_n;
    bool tie = false;
    for (int base = 0; base < n; base += 32) {
        int i = base + lane;
        dd v = {i < n ? w[i] : 0.0, 0.0};
        dd incl = dd_add(carry, wscan_dd(v, lane));
        carry = {__shfl_sync(FULL, incl.hi, 31), __shfl_sync(FULL, incl.lo, 31)};
        dd x = dd_add(dd_mul_d(incl, dn), dd_neg(u0));
        double frac;
        long long C = dd_floor(x, frac) + 1;
        if (i < n && (frac < 1e-20 || frac > 1.0 - 1e-20)) tie = true;
        long long Cp = __shfl_up_sync(FULL, C, 1);
        if (lane == 0) Cp = prevC;
        if (i < n) cnt[i] = (int)(C - Cp);
        prevC = __shfl_sync(FULL, C, 31);
    }
    tie = __any_sync(FULL, tie);
    if (tie) {
        if (lane == 0) {
            q128 dnq = q128_from_int(count_n);
            q128 u = q128_div(q128_add(q128_from_double(u_hi), q128_from_double(u_lo)), dnq);
            for (int i = 0; i < n; ++i) {
                q128 wi = q128_from_double(w[i]);
                long long aq = q128_floor(q128_mul(q128_sub(wi, u), dnq)) + 1;
                cnt[i] = (int)aq;
                u = q128_sub(q128_add(u, q128_div(q128_from_int(aq), dnq)), wi);
            }
        }
        __syncwarp();
        long long t = 0;
        for (int i = lane; i < n; i += 32) t += cnt[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
        return t;
    }
    return prevC;
}

template <typename T, int RT>
__device__ __forceinline__ void warp_gemm(const T *__restrict__ Mcol, const T *__restrict__ X, int rg, int cg,
                                          T acc[RT][CTW]) {
    constexpr int DP = RGW * RT;
#pragma unroll
    for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int q = 0; q < CTW; ++q) acc[i][q] = T(0);
    const T *mp = Mcol + rg * RT;
    const T *xp = X + cg * CTW;
#pragma unroll 4
    for (int k = 0; k < DP; ++k) {
        T mv[RT], xv[CTW];
#pragma unroll
        for (int i = 0; i < RT; ++i) mv[i] = mp[k * DP + i];
#pragma unroll
        for (int q = 0; q < CTW; ++q) xv[q] = xp[k * CW + q];
#pragma unroll
        for (int i = 0; i < RT; ++i)
#pragma unroll
            for (int q = 0; q < CTW; ++q) acc[i][q] = fma(mv[i], xv[q], acc[i][q]);
    }
}

// ---- shared memory of one group
//
// CUDA-core engine: M (DP x DP, T), W double-buffered DP x 8 slot tiles.
// tcgen05 engine: A hi/lo (128 x DP BF16 core-matrix operands), B hi/lo
// (S x DP), the FP32 end-point tile Xf (DP x S) aliasing B.
// Warp-MMA engine: A hi/lo (DP x DP, row stride DP+8), two B buffers hi/lo
// (DP x S, row stride S+8), FP32 tiles X, P, XC (DP x S, row stride S+1);
// the end-point offsets tile aliases the idle B buffer.
// All: per-dimension T and double arrays, per-slot state, scratch.
template <typename T, int RT, int ENG>
struct Layout {
    static constexpr int DP = RGW * RT;
    // warp-MMA engine beyond 128 dimensions: the stage matrix (4 DP^2 bytes as
    // BF16 hi + lo) no longer fits in shared memory; it is kept in global memory
    // in fragment order and streamed through a per-warp ring, and the FP32 Gram
    // matrix of the end-point energies is read from global memory
    static constexpr bool AGL = ENG == ENG_MMA && DP > 128;
    // global-matrix engine: GL_S slots per group of 16 warps (16; 8 for FP64
    // beyond 512 dimensions, where a thread's positions, momenta and products
    // would exceed its registers); a thread owns GL_SPT slots of one slot group
    // and DP / (512 * GL_SPT / GL_S) rows
    static constexpr int GL_S = (sizeof(T) == 8 && DP > 512) ? 8 : 16;
    static constexpr int GL_SPT = DP <= 256 ? 8 : (GL_S == 8 ? 8 : 16);
    // columns of the stage matrix in flight per thread (gl_gemm's ring): a
    // ring slot holds the thread's DP / RP entries of one column, and the
    // ring of the whole group takes GL_RING * DP * (GL_S / GL_SPT) entries
    static constexpr int GL_RING = (sizeof(T) == 8 && DP > 512) ? 6 : 16;
    static constexpr size_t GL_RING_BYTES = (size_t)GL_RING * DP * (GL_S / GL_SPT) * sizeof(T);
    static constexpr int S = ENG == ENG_CC ? CW : ENG == ENG_GL ? GL_S : ENG == ENG_MMAQ ? 1024 / DP
                             : (AGL ? 4096 / DP : 2048 / DP);   // slots per warp (CC) / group
    // the FP32 Gram matrix of the end-point energies: in shared memory (warp
    // MMA up to 128 dimensions) or read from global memory (AGL, MMAQ)
    static constexpr bool A32_GLOBAL = AGL || ENG == ENG_MMAQ;
    static constexpr int RING = 6;                       // streamed k-tiles in flight per warp
    static constexpr uint32_t LBO_A = 2048;              // tcgen05: 128 rows x 16 B per k block
    static constexpr uint32_t LBO_B = 16 * S + 16;       // tcgen05: S rows x 16 B per k block, padded
    static constexpr size_t A_BYTES = ENG == ENG_TC ? (size_t)LBO_A * (DP / 8) : AGL ? 0 : (size_t)DP * (DP + 8) * 2;
    static constexpr size_t B_BYTES = ENG == ENG_TC ? (size_t)LBO_B * (DP / 8) : (size_t)DP * (S + 8) * 2;
    static constexpr int AST = DP + 8, BST = S + 8, TS = S + 1;   // warp-MMA row strides (elements)
    static constexpr size_t TILE_BYTES = (size_t)DP * TS * sizeof(float);
    // m-tiles per warp of the warp-MMA step with W warps
    __host__ __device__ static constexpr int mtiles_per_warp(int W) {
        return (DP / 16) * (S / 8) / W > S / 8 ? (DP / 16) / W : 1;
    }
    // streamed A ring: RING slots x m-tiles x (hi, lo) x 32 lanes x 16 bytes per warp
    __host__ __device__ static constexpr size_t ring_bytes(int W) {
        return AGL ? (size_t)W * RING * mtiles_per_warp(W) * 2 * 32 * 16 : 0;
    }
    __host__ __device__ static size_t engine_bytes(int W) {
        if (ENG == ENG_GL) return (size_t)DP * S * sizeof(T) + GL_RING_BYTES;  // step operand [row][slot], ring
        if (ENG == ENG_TC) return 2 * A_BYTES + 2 * B_BYTES;   // the end-point tile Xf aliases B
        if (is_mma(ENG))   // + the FP32 Gram matrix for the end-point energies (or the A ring)
            return 2 * A_BYTES + 4 * B_BYTES + 3 * TILE_BYTES +
                   (AGL ? ring_bytes(W) : A32_GLOBAL ? 0 : (size_t)DP * DP * sizeof(float));
        return (size_t)DP * DP * sizeof(T) + (size_t)W * 2 * DP * CW * sizeof(T);
    }
    __host__ __device__ static int slots(int W) { return ENG == ENG_CC ? W * CW : S; }
    // per-slot partial sums of the end-point energies: 5 x 32 W floats (warp MMA)
    // or 5 x 32 max(W, 4) doubles (tcgen05)
    __host__ __device__ static size_t red_bytes(int W) {
        if (ENG == ENG_GL)   // per-warp, per-slot partial sums of 5 quantities (also 32 W floats of moments)
            return (size_t)5 * W * S * sizeof(double) > (size_t)32 * W * sizeof(float)
                       ? (size_t)5 * W * S * sizeof(double) : (size_t)32 * W * sizeof(float);
        return is_mma(ENG) ? (size_t)5 * 32 * W * sizeof(float) : (size_t)5 * 32 * (W > 4 ? W : 4) * sizeof(double);
    }
    __host__ __device__ static size_t bytes(int W) {
        size_t b = engine_bytes(W) + (size_t)7 * DP * sizeof(T) + (size_t)6 * DP * sizeof(double) +
                   (size_t)slots(W) * (5 * sizeof(double) + 5 * sizeof(int)) + (size_t)(4 * W + 8) * sizeof(double);
        if (ENG != ENG_CC) b += red_bytes(W) + 64;   // reductions, masks, mbarrier
        return (b + 127) & ~(size_t)127;
    }
};

}  // namespace

template <typename T, int RT, int ENG, int WG>
__device__ __forceinline__ void group_body(const MeshDev &m, const InnerArgs &a, Group &grp, int th,
                                           unsigned char *smem, uint32_t tmem_base) {
    using L_ = Layout<T, RT, ENG>;
    constexpr int DP = L_::DP;
    constexpr bool MIXED = std::is_same<T, float>::value;
    constexpr bool TC = ENG == ENG_TC;
    static_assert(ENG == ENG_CC || ENG == ENG_GL || MIXED, "tensor-core engines are MIXED only");
    const int lane = grp.lane;
    const int N = a.N, D = a.D, NP2 = a.NP2;
    const int rg = lane & 15, cg = lane >> 4, gt = grp.gt, gnt = grp.nt, wl = grp.wl, W = grp.W;
    const int NS = L_::slots(W);

    // ---- shared memory carve-up
    unsigned char *sp = smem;
    T *Msm = nullptr, *Xw0 = nullptr, *Xw1 = nullptr;
    unsigned char *Ahi = nullptr, *Alo = nullptr, *Bhi = nullptr, *Blo = nullptr;
    float *Xf = nullptr, *tX = nullptr, *tP = nullptr, *tXC = nullptr, *tA32 = nullptr;
    uint4 *aring = nullptr;
    if constexpr (is_mma(ENG)) {
        // B buffer b: hi at Bhi + 2*b*B_BYTES, lo B_BYTES after it
        Ahi = sp; Alo = Ahi + L_::A_BYTES; Bhi = Alo + L_::A_BYTES; Blo = Bhi + L_::B_BYTES;
        tX = (float *)(Bhi + 4 * L_::B_BYTES);
        tP = (float *)((unsigned char *)tX + L_::TILE_BYTES);
        tXC = (float *)((unsigned char *)tP + L_::TILE_BYTES);
        if constexpr (L_::AGL) aring = (uint4 *)((unsigned char *)tXC + L_::TILE_BYTES);
        else if constexpr (!L_::A32_GLOBAL) tA32 = (float *)((unsigned char *)tXC + L_::TILE_BYTES);
        static_assert(2 * L_::B_BYTES >= L_::TILE_BYTES, "offset tile must fit in one B buffer");
    } else if constexpr (ENG == ENG_GL) {
        Msm = nullptr;
        Xw0 = (T *)sp;                        // step operand [row][slot]
        Xw1 = Xw0 + (size_t)DP * L_::S;       // gl_gemm's per-thread column ring
    } else if constexpr (TC) {
        Ahi = sp; Alo = Ahi + L_::A_BYTES; Bhi = Alo + L_::A_BYTES; Blo = Bhi + L_::B_BYTES;
        Xf = (float *)Bhi;   // written at the last leapfrog step, after the last MMA read B
        static_assert(2 * L_::B_BYTES >= (size_t)DP * L_::S * sizeof(float), "Xf must fit in B");
    } else {
        Msm = (T *)sp;
        Xw0 = Msm + DP * DP + (size_t)wl * 2 * DP * CW;
        Xw1 = Xw0 + DP * CW;
    }
    sp += L_::engine_bytes(W);
    T *tcov = (T *)sp, *tmean = tcov + DP, *tcv = tmean + DP, *tisc = tcv + DP;
    T *tvg = tisc + DP, *tvh = tvg + DP, *ticov = tvh + DP;   // MIXED end-point terms in T
    double *vb = (double *)(ticov + DP);
    double *vcov = vb + DP, *vmean = vcov + DP, *vg = vmean + DP, *vh = vg + DP, *vc = vh + DP;
    double *sdall = vc + DP;                                   // NS * 5 doubles
    int *siall = (int *)(sdall + (size_t)NS * 5);              // NS * 5 ints
    double *gscr = (double *)(siall + (size_t)NS * 5 + ((NS * 5) & 1));
    int *gint = (int *)(gscr + 4 * W);   // [0] queue head, [2] status, [3] wait gave up
    grp.scr = gscr;
    // per-warp (CC) or per-group (TC) slot state
    const int sbase = ENG != ENG_CC ? 0 : wl * CW;
    double *sL = sdall + sbase, *sP = sL + NS, *spost = sP + NS, *sham = spost + NS, *sdt = sham + NS;
    int *spar = siall + sbase, *sj = spar + NS, *sjend = sj + NS, *sfresh = sjend + NS, *sblown = sfresh + NS;
    double *red = nullptr;
    unsigned long long *masks = nullptr;   // [0] fresh, [1] active, [2] blown, [3] accepted
    uint64_t *mbar = nullptr;
    if constexpr (ENG != ENG_CC) {
        red = (double *)(gint + 8);   // per-slot partial sums
        masks = (unsigned long long *)((unsigned char *)red + L_::red_bytes(W));
        mbar = (uint64_t *)(masks + 4);
    }

    const double *Ath = a.A + (size_t)th * D * D;
    const double *bth = a.b + (size_t)th * D;
    const double dsd = a.dsd[th];
    const ThetaAux ax = a.aux[th];
    const double alpha2 = ax.alpha2, lconst = ax.lconst;
    const double *lv = a.lval + (size_t)th * m.nrow * 9;
    const double *llv = a.llval + (size_t)th * m.ll_nnz;
    const uint64_t stream = a.streams[th];
    double *parts = a.parts + (size_t)th * N * D, *pnew = a.parts_new + (size_t)th * N * D;
    double *Lc = a.dbuf + (size_t)th * 9 * N, *Pc = Lc + N, *Ln = Lc + 2 * N, *Pn = Lc + 3 * N, *w = Lc + 4 * N;
    double *dtau = Lc + 5 * N, *dtn = Lc + 6 * N, *score = Lc + 7 * N;
    int *cnt = a.ibuf + (size_t)th * 4 * NP2, *ids = cnt + NP2, *keys = cnt + 2 * NP2, *sub = cnt + 3 * NP2;
    float *A32 = a.A32 ? a.A32 + (size_t)th * D * D : nullptr;
    const T mx = (T)a.max_slip;
    int status = 0;
    uint32_t phase = 0;   // TC: parity of the next mbarrier phase

    if (gt == 0) { gint[2] = 0; gint[3] = 0; }
    if constexpr (TC) {
        if (gt == 0) tc::mbar_init(mbar, 1);
    }
    for (int i = gt; i < DP; i += gnt) vb[i] = i < D ? bth[i] : 0.0;
    for (int k = gt; k < N; k += gnt) dtau[k] = exp(-5.0);
    float *lv32 = a.lv32 ? a.lv32 + (size_t)th * m.nrow * 9 : nullptr;
    float *ll32 = a.ll32 ? a.ll32 + (size_t)th * m.ll_nnz : nullptr;
    float *wf = (float *)(Lc + 8 * N);   // MIXED: FP32 copy of the normalised weights
    if constexpr (is_mma(ENG)) {
        if constexpr (L_::A32_GLOBAL) {
            for (int e = gt; e < D * D; e += gnt) A32[e] = (float)Ath[e];
        } else {
            for (int e = gt; e < DP * DP; e += gnt) {
                const int k = e / DP, r = e % DP;
                tA32[e] = (k < D && r < D) ? (float)Ath[(size_t)k * D + r] : 0.0f;
            }
        }
        for (int e = gt; e < m.nrow * 9; e += gnt) lv32[e] = (float)lv[e];
        for (int e = gt; e < m.ll_nnz; e += gnt) ll32[e] = (float)llv[e];
    } else if (MIXED) {
        for (int e = gt; e < D * D; e += gnt) A32[e] = (float)Ath[e];
    }
    grp.sync();

    // initial likelihoods and priors, FP64 Gram form (smc_slip.f90:273-286)
    for (int k = wl; k < N; k += W) {
        const double *x = parts + (size_t)k * D;
        double qa = 0.0, bx = 0.0, pr = 0.0;
        for (int i = lane; i < D; i += 32) {
            double t = 0.0;
            for (int j2 = 0; j2 < D; ++j2) t += Ath[(size_t)j2 * D + i] * x[j2];
            qa += x[i] * t;
            bx += vb[i] * x[i];
        }
        for (int r = lane; r < m.nrow; r += 32) {
            double t = 0.0;
            for (int q = 0; q < 9; ++q) {
                int c = m.l_col[r * 9 + q];
                if (c >= 0) t += lv[(size_t)r * 9 + q] * x[c];
            }
            pr += t * t / (2.0 * alpha2);
        }
        qa = wsum(qa);
        bx = wsum(bx);
        pr = wsum(pr);
        if (lane == 0) {
            Lc[k] = (qa - 2.0 * bx + dsd) / 2.0 + lconst;
            Pc[k] = pr;
        }
    }
    grp.sync();
    // A geometry whose initial population has a non-finite likelihood or prior
    // (a non-finite theta or observation, a degenerate plane) is abandoned with
    // SMCGPU_ST_NONFINITE and neglog = NaN: the reference would carry the NaN
    // through every stage.
    bool nonfinite = false;
    {
        double bad = 0.0;
        for (int k = gt; k < N; k += gnt) bad += (isfinite(Lc[k]) && isfinite(Pc[k])) ? 0.0 : 1.0;
        nonfinite = grp.sum(bad) > 0.0;
    }

    double gamma = 0.0, neglog = 0.0, log_up = 0.0, log_lo = -1e1;
    double ntraj = 0.0;   // HMC trajectories run (tuning and sampling)
    int iter = 1;
    while (!nonfinite && 1.0 - gamma > 10e-8) {
        // ---- next tempering exponent (smc_slip.f90:314-387)
        double lmin = 1e300;
        for (int k = gt; k < N; k += gnt) lmin = fmin(lmin, Lc[k]);
        lmin = grp.min(lmin);
        const double gprev = gamma;
        double lower = gprev, upper = 1.0, err = 1.0, g = 1.0;
        int bcnt = 0;
        const double tol = MIXED ? 1e-6 : 1e-10;
        // MIXED: this thread's first LR likelihood offsets held in registers
        constexpr int LR = 4;
        float lr[LR];
        if (MIXED) {
#pragma unroll
            for (int q = 0; q < LR; ++q) {
                const int k = gt + q * gnt;
                lr[q] = k < N ? (float)(Lc[k] - lmin) : 0.0f;
            }
        }
        while (err > tol) {
            g = (lower + upper) / 2.0;
            double dg = g - gprev, cv;
            if (MIXED) {
                // weights in (0, 1] summed in FP32: the CV target (2) keeps
                // s2/N - mean^2 well away from cancellation
                float dgf = (float)dg;
                float ps = 0.0f, ps2 = 0.0f;
#pragma unroll
                for (int q = 0; q < LR; ++q)
                    if (gt + q * gnt < N) {
                        float wk = expf(-dgf * lr[q]);
                        ps += wk;
                        ps2 = fmaf(wk, wk, ps2);
                    }
                for (int k = gt + LR * gnt; k < N; k += gnt) {
                    float wk = expf(-dgf * (float)(Lc[k] - lmin));
                    ps += wk;
                    ps2 = fmaf(wk, wk, ps2);
                }
                grp.sum2f(ps, ps2);
                const float invn = 1.0f / (float)N, meanf = ps * invn;
                cv = (double)(sqrtf(fmaxf(ps2 * invn - meanf * meanf, 0.0f)) / meanf);
            } else {
                double ps = 0.0;
                for (int k = gt; k < N; k += gnt) {
                    double wk = exp(-dg * (Lc[k] - lmin));
                    w[k] = wk;
                    ps += wk;
                }
                double mean = grp.sum(ps) / N;
                double pv = 0.0;
                for (int k = gt; k < N; k += gnt) {
                    double dv = w[k] - mean;
                    pv += dv * dv;
                }
                cv = sqrt(grp.sum(pv) / N) / mean;
            }
            if (cv > a.cv) upper = g; else lower = g;
            err = fabs(cv - a.cv);
            if (fabs(g - 1.0) < 1e-10) break;
            if (MIXED && upper - lower < 1e-12 * fmax(1.0, g)) break;
            if (++bcnt > 2000) { status |= SMCGPU_ST_BISECT_CAP; break; }
        }
        double dg = g - gprev, ps = 0.0;
        for (int k = gt; k < N; k += gnt) {
            double wk = exp(-dg * (Lc[k] - lmin));
            w[k] = wk;
            ps += wk;
        }
        double ev = grp.sum(ps) / N;
        double inc = -log(ev) + dg * lmin;
        if (!isfinite(inc)) {   // the weights of this stage are not finite
            nonfinite = true;
            break;
        }
        gamma = g;
        neglog += inc;
        if (gt == 0 && a.trace_gamma) {
            a.trace_gamma[(size_t)th * (a.max_stages + 2) + iter - 1] = gamma;
            a.trace_inc[(size_t)th * (a.max_stages + 2) + iter - 1] = inc;
        }
        if (iter > a.max_stages) {
            neglog = 1e10;
            status |= SMCGPU_ST_STAGE_CAP;
            break;
        }
        // ---- normalise, weighted mean and diagonal covariance (smc_slip.f90:465-570)
        {
            dd p2 = {0.0, 0.0};
            for (int k = gt; k < N; k += gnt) p2 = dd_add_d(p2, w[k]);
            dd sw = grp.sum_dd(p2);
            for (int k = gt; k < N; k += gnt) {
                w[k] = dd_div_into_w(w[k], sw);
                if (MIXED) wf[k] = (float)w[k];
            }
            grp.sync();
        }
        if constexpr (MIXED && ENG != ENG_CC && ENG != ENG_GL) {
            // thread (d, kp) sums particles k = kp, kp + KP, ...; partials in FP32
            const int KP = gnt / DP, d = gt % DP, kp = gt / DP;
            float *fs = (float *)red;
            float md = 0.0f;
            if (kp < KP && d < D)
                for (int k = kp; k < N; k += KP) md = fmaf(wf[k], f32_of_f32valued(parts[(size_t)k * D + d]), md);
            fs[gt] = md;
            grp.sync();
            if (gt < DP) {
                float t = 0.0f;
                for (int q = 0; q < KP; ++q) t += fs[q * DP + gt];
                vmean[gt] = gt < D ? (double)t : 0.0;
            }
            grp.sync();
            const float mu = (float)vmean[d];
            float cd = 0.0f;
            if (kp < KP && d < D)
                for (int k = kp; k < N; k += KP) {
                    const float di = f32_of_f32valued(parts[(size_t)k * D + d]) - mu;
                    cd = fmaf(wf[k] * di, di, cd);
                }
            fs[gt] = cd;
            grp.sync();
            if (gt < DP) {
                float t = 0.0f;
                for (int q = 0; q < KP; ++q) t += fs[q * DP + gt];
                vcov[gt] = gt >= D ? 1.0 : (fabsf(t) < 1e-3f ? 1e-3 : (double)t);
            }
        } else
        for (int d = gt; d < DP; d += gnt) {
            if (d >= D) { vmean[d] = 0.0; vcov[d] = 1.0; continue; }
            if (!MIXED) {
                dd md = {0.0, 0.0};
                for (int k = 0; k < N; ++k) md = dd_add_d(md, w[k] * parts[(size_t)k * D + d]);
                double mean = md.hi + md.lo;
                dd cd = {0.0, 0.0};
                for (int k = 0; k < N; ++k) {
                    double di = parts[(size_t)k * D + d] - mean;
                    cd = dd_add_d(cd, w[k] * di * di);
                }
                double cv = cd.hi + cd.lo;
                vmean[d] = mean;
                vcov[d] = fabs(cv) < 1e-3 ? 1e-3 : cv;
            } else {
                float md = 0.0f;
                for (int k = 0; k < N; ++k) md = fmaf((float)w[k], (float)parts[(size_t)k * D + d], md);
                float cd = 0.0f;
                for (int k = 0; k < N; ++k) {
                    float di = (float)parts[(size_t)k * D + d] - md;
                    cd = fmaf((float)w[k] * di, di, cd);
                }
                vmean[d] = md;
                vcov[d] = fabsf(cd) < 1e-3f ? 1e-3 : (double)cd;
            }
        }
        // ---- resampling counts (smc_slip.f90:572-589) and child offsets (warp 0)
        if (wl == 0) {
            double uh, ul;
            rng_quad_uniform(a.seed, stream, RNG_RESAMPLE, iter, uh, ul);
            warp_counts(w, N, N, uh, ul, cnt, lane);
            __syncwarp();
            int carry = 0;
            for (int base = 0; base < N; base += 32) {
                int k = base + lane, tot;
                int v = k < N ? cnt[k] : 0;
                int ex = wexscan(v, lane, tot);
                if (k < N) ids[k] = carry + ex;
                carry += tot;
            }
        }
        // ---- stage matrix
        if constexpr (L_::AGL) {
            // M = gamma A + L^T L / alpha^2 in FP32 from the global FP32 copy of A,
            // split into BF16 hi + lo and stored in m16n8k16 A-fragment order:
            // [m-tile][k-tile][hi, lo][lane] x 16 bytes, register j of lane (g, t4)
            // holding row 16 mt + g + 8 (j & 1), columns 16 kt + 2 t4 + 8 (j >> 1) + {0, 1}
            constexpr int KT = DP / 16;
            const float gf = (float)gamma, ia2 = (float)(1.0 / alpha2);
            uint4 *fr = a.afrag + (size_t)th * (DP * DP / 4);
            for (int q = gt; q < KT * KT * 32; q += gnt) {
                const int ln = q & 31, tile = q >> 5, mt = tile / KT, kt = tile % KT;
                const int g8 = ln >> 2, t4 = ln & 3;
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int i = 16 * mt + g8 + 8 * (j & 1), k0 = 16 * kt + 2 * t4 + 8 * (j >> 1);
                    float v[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int k = k0 + h;
                        float vv = 0.0f;
                        if (i < D && k < D) {
                            vv = gf * A32[(size_t)k * D + i];
                            for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e)
                                if (m.ll_col[e] == k) { vv += ll32[e] * ia2; break; }
                        }
                        v[h] = vv;
                    }
                    const __nv_bfloat162 hi = __floats2bfloat162_rn(v[0], v[1]);
                    const __nv_bfloat162 lo = __floats2bfloat162_rn(v[0] - __low2float(hi), v[1] - __high2float(hi));
                    hw[j] = bf16x2_bits(hi);
                    lw[j] = bf16x2_bits(lo);
                }
                fr[(size_t)(2 * tile) * 32 + ln] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                fr[(size_t)(2 * tile + 1) * 32 + ln] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        } else if constexpr (is_mma(ENG)) {
            // M = gamma A + L^T L / alpha^2 in FP32 (A from the FP32 copy in shared
            // memory, or in global memory for MMAQ), split into BF16 hi + lo,
            // row-major with row stride DP+8;
            // TPR threads per row, KC consecutive columns each
            const float gf = (float)gamma, ia2 = (float)(1.0 / alpha2);
            const int TPR = gnt / DP, KC = DP / TPR;
            for (int q = gt; q < DP * TPR; q += gnt) {
                const int i = q / TPR, k0 = (q % TPR) * KC;
                int e = i < D ? m.ll_ptr[i] : 0;
                const int e1 = i < D ? m.ll_ptr[i + 1] : 0;
                while (e < e1 && m.ll_col[e] < k0) ++e;
                __nv_bfloat16 *rh = (__nv_bfloat16 *)Ahi + (size_t)i * L_::AST;
                __nv_bfloat16 *rl = (__nv_bfloat16 *)Alo + (size_t)i * L_::AST;
                for (int k = k0; k < k0 + KC; ++k) {
                    float v = 0.0f;
                    if (i < D && k < D) {
                        if constexpr (L_::A32_GLOBAL) v = gf * A32[(size_t)k * D + i];
                        else v = gf * tA32[k * DP + i];
                        if (e < e1 && m.ll_col[e] == k) { v += ll32[e] * ia2; ++e; }
                    }
                    tc::split_bf16(v, rh[k], rl[k]);
                }
            }
        } else if constexpr (ENG == ENG_GL) {
            // M = gamma A + L^T L / alpha^2 in global memory, column-major, in T
            // (MIXED: from the FP32 copy of A, as the warp-MMA engine)
            T *Mw = (T *)a.mgl + (size_t)th * D * D;
            if constexpr (MIXED) {
                const float gf = (float)gamma;
                for (int e = gt; e < D * D; e += gnt) Mw[e] = gf * A32[e];
            } else {
                for (int e = gt; e < D * D; e += gnt) Mw[e] = (T)(gamma * Ath[e]);
            }
            grp.sync();
            const float ia2 = (float)(1.0 / alpha2);
            for (int i = gt; i < D; i += gnt)
                for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) {
                    const int k = m.ll_col[e];
                    if constexpr (MIXED) Mw[(size_t)k * D + i] += (float)llv[e] * ia2;
                    else Mw[(size_t)k * D + i] = (T)((double)Mw[(size_t)k * D + i] + llv[e] / alpha2);
                }
        } else if constexpr (TC) {
            // row t of the 128-row A operand is M's row t % DP, split into BF16 hi + lo
            const int i = gt % DP;
            int e = i < D ? m.ll_ptr[i] : 0;
            const int e1 = i < D ? m.ll_ptr[i + 1] : 0;
            for (int k = 0; k < DP; ++k) {
                double v = 0.0;
                if (i < D && k < D) {
                    v = gamma * Ath[(size_t)k * D + i];
                    while (e < e1 && m.ll_col[e] < k) ++e;
                    if (e < e1 && m.ll_col[e] == k) v += llv[e] / alpha2;
                }
                __nv_bfloat16 hi, lo;
                tc::split_bf16((float)v, hi, lo);
                const uint32_t off = tc::core_offset(gt, k, L_::LBO_A);
                *(__nv_bfloat16 *)(Ahi + off) = hi;
                *(__nv_bfloat16 *)(Alo + off) = lo;
            }
        } else {
            for (int e = gt; e < DP * DP; e += gnt) {
                int i = e % DP, k = e / DP;
                Msm[e] = (i < D && k < D) ? (T)(gamma * Ath[(size_t)k * D + i]) : T(0);
            }
            grp.sync();
            for (int i = gt; i < D; i += gnt)
                for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) {
                    int k = m.ll_col[e];
                    Msm[k * DP + i] = (T)((double)Msm[k * DP + i] + llv[e] / alpha2);
                }
        }
        // ---- centring terms (MIXED): g = A sbar - b, h = L^T L sbar / alpha^2
        double Lbar = 0.0, Pbar = 0.0;
        if (MIXED) {
            double qa = 0.0, bx = 0.0, pr = 0.0;
            for (int i = gt; i < DP; i += gnt) {
                double gi = 0.0, hi = 0.0, t = 0.0;
                if (i < D) {
                    for (int k = 0; k < D; ++k) t += Ath[(size_t)k * D + i] * vmean[k];
                    gi = t - vb[i];
                    for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) hi += llv[e] * vmean[m.ll_col[e]];
                    hi /= alpha2;
                    qa += vmean[i] * t;
                    bx += vb[i] * vmean[i];
                }
                vg[i] = gi;
                vh[i] = hi;
                vc[i] = gamma * gi + hi;
            }
            for (int r = gt; r < m.nrow; r += gnt) {
                double t = 0.0;
                for (int q = 0; q < 9; ++q) {
                    int c = m.l_col[r * 9 + q];
                    if (c >= 0) t += lv[(size_t)r * 9 + q] * vmean[c];
                }
                pr += t * t / (2.0 * alpha2);
            }
            qa = grp.sum(qa);
            bx = grp.sum(bx);
            pr = grp.sum(pr);
            Lbar = (qa - 2.0 * bx + dsd) / 2.0 + lconst;
            Pbar = pr;
        }
        grp.sync();
        for (int i = gt; i < DP; i += gnt) {
            tcov[i] = (T)vcov[i];
            tmean[i] = (T)vmean[i];
            tcv[i] = MIXED ? (T)vc[i] : (T)(gamma * vb[i]);
            tisc[i] = (T)(1.0 / sqrt(vcov[i]));
            tvg[i] = (T)vg[i];
            tvh[i] = (T)vh[i];
            ticov[i] = (T)(1.0 / vcov[i]);
        }
        grp.sync();

        // ---- HMC passes: tuning (every tf-th parent, smc_slip.f90:919-1214),
        // then sampling (smc_slip.f90:591-730)
        for (int pass = 0; pass < 2; ++pass) {
            const bool tuning = pass == 0;
            const uint32_t P_MOM = tuning ? RNG_TUNE_MOM : RNG_SMP_MOM;
            const uint32_t P_MH = tuning ? RNG_TUNE_MH : RNG_SMP_MH;
            double nql = 0.0, ntl = 0.0;
            for (int k = gt; k < NP2; k += gnt) {
                bool ok = k < N && cnt[k] > 0 && (!tuning || k % a.tf == 0);
                keys[k] = ok ? (int)(((unsigned)(N - cnt[k]) << 16) | (unsigned)k) : 0x7fffffff;
                nql += ok;
                ntl += ok ? cnt[k] : 0;   // one trajectory per child of a queued parent
            }
            grp.sum2(nql, ntl);
            const int nq = (int)nql;
            ntraj += ntl;
            grp.sync();
            for (int size = 2; size <= NP2; size <<= 1)
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int i = gt; i < NP2; i += gnt) {
                        int jx = i ^ stride;
                        if (jx > i) {
                            int ka = keys[i], kb = keys[jx];
                            bool up = (i & size) == 0;
                            if ((ka > kb) == up) { keys[i] = kb; keys[jx] = ka; }
                        }
                    }
                    grp.sync();
                }
            if (tuning && nq == 0) continue;   // no tuned child (smc_slip.f90:993-995)
            if (tuning) {
                for (int q = gt; q < nq; q += gnt) {
                    int k = keys[q] & 0xffff;
                    for (int jj = ids[k]; jj < ids[k] + cnt[k]; ++jj) {
                        double ld = rng_uniform(a.seed, stream, RNG_TUNE_DTAU, iter, jj, 0);
                        ld = log_lo + ld * (log_up - log_lo);
                        dtau[jj] = exp(ld);
                    }
                }
            }
            if constexpr (is_mma(ENG)) {
                // ================= warp-MMA engine: S slots per group.
                // Step layout: warp wl owns m-tiles mt0.. (16 dimensions each) x
                // n-tiles nt0.. (8 slots each); lane (g, t4) holds rows 16 mt + g and
                // + 8 of slots 8 nt + 2 t4 and + 1 (the m16n8 accumulator layout).
                // Chain-start / end-point layout: thread (cs = gt % S, part = gt / S)
                // handles slot cs on dimensions part, part + NPART, ...
                constexpr int S = L_::S, NT = S / 8, NTH = 32 * WG, NPART = NTH / S;
                constexpr int PPW = (DP / 16) * NT / WG;   // (m-tile, n-tile) pairs per warp
                constexpr int MTW = PPW > NT ? PPW / NT : 1, NTW = PPW / MTW;
                constexpr int AST = L_::AST, BST = L_::BST, TS = L_::TS, KT = DP / 16;
                static_assert(MTW * NTW * WG == (DP / 16) * NT, "every (m-tile, n-tile) pair has one owner");
                const int g = lane >> 2, t4 = lane & 3;
                const int mt0 = (wl * PPW) / NT, nt0 = (wl * PPW) % NT;
                const int cs = gt % S, part = gt / S;
                const __nv_bfloat16 *Ah = (const __nv_bfloat16 *)Ahi, *Al = (const __nv_bfloat16 *)Alo;
                unsigned *m32 = (unsigned *)masks;   // halves: [0,1] fresh [2,3] active [4,5] blown [6,7] accepted
                float cov_l[MTW][2], mean_l[MTW][2], cv_l[MTW][2];
                bool live_l[MTW][2];
#pragma unroll
                for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int r = 16 * (mt0 + aa) + g + 8 * h;
                        cov_l[aa][h] = (float)tcov[r];
                        mean_l[aa][h] = (float)tmean[r];
                        cv_l[aa][h] = (float)tcv[r];
                        live_l[aa][h] = r < D;
                    }
                float x[MTW][NTW][4], p[MTW][NTW][4], dts[NTW][2];
                const float imx = 1.0f / (float)mx;
                // this warp's rows of M as A fragments (hi, lo): held in registers
                // for the whole pass when they are few, else loaded every step
                constexpr bool AREG = MTW * KT <= 4;
                constexpr int KTR = AREG ? KT : 1;
                uint32_t fah[MTW][KTR][4], fal[MTW][KTR][4];
                auto load_a = [&](int kt, int slot) {
#pragma unroll
                    for (int aa = 0; aa < MTW; ++aa) {
                        const int row = 16 * (mt0 + aa) + (lane & 7) + 8 * ((lane >> 3) & 1);
                        const int col = 16 * kt + 8 * (lane >> 4);
                        ldsm_x4(fah[aa][slot], Ah + row * AST + col);
                        ldsm_x4(fal[aa][slot], Al + row * AST + col);
                    }
                };
                if constexpr (AREG) {
#pragma unroll
                    for (int kt = 0; kt < KT; ++kt) load_a(kt, kt);
                }
                // streamed A (beyond 128 dimensions): k-tile kt of this warp's m-tiles
                // goes to ring slot kt % RING; every lane copies and later reads only
                // its own 16-byte fragments, so no warp barrier is needed
                constexpr int RING = L_::RING;
                const uint4 *afr = L_::AGL ? a.afrag + (size_t)th * (DP * DP / 4) : nullptr;
                uint4 *wring = L_::AGL ? aring + (size_t)wl * RING * MTW * 64 : nullptr;
                auto issue_a = [&](int kt) {
                    if (kt < KT) {
#pragma unroll
                        for (int aa = 0; aa < MTW; ++aa) {
                            const uint4 *src = afr + (size_t)(2 * ((mt0 + aa) * KT + kt)) * 32 + lane;
                            uint4 *dst = wring + (size_t)(2 * ((kt % RING) * MTW + aa)) * 32 + lane;
                            cp_async16(dst, src);
                            cp_async16(dst + 32, src + 32);
                        }
                    }
                    cp_async_commit();   // an empty group past the last k-tile keeps the count uniform
                };
                // offsets from the stage mean of the lane's entries -> BF16 hi/lo operand buffer
                auto write_b = [&](int buf) {
                    __nv_bfloat16 *bh = (__nv_bfloat16 *)(Bhi + 2 * (size_t)buf * L_::B_BYTES);
                    __nv_bfloat16 *bl = (__nv_bfloat16 *)(Bhi + (2 * (size_t)buf + 1) * L_::B_BYTES);
#pragma unroll
                    for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                        for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const int r = 16 * (mt0 + aa) + g + 8 * h, c0 = 8 * (nt0 + bb) + 2 * t4;
                                // rows beyond D hold x = 0 and mean 0: their offsets are 0
                                const float d0 = x[aa][bb][2 * h] - mean_l[aa][h];
                                const float d1 = x[aa][bb][2 * h + 1] - mean_l[aa][h];
                                const __nv_bfloat162 hi = __floats2bfloat162_rn(d0, d1);
                                const __nv_bfloat162 lo = __floats2bfloat162_rn(d0 - __low2float(hi), d1 - __high2float(hi));
                                *(uint32_t *)(bh + r * BST + c0) = bf16x2_bits(hi);
                                *(uint32_t *)(bl + r * BST + c0) = bf16x2_bits(lo);
                            }
                };
                if (gt == 0) gint[0] = 0;
                if (gt < 2) m32[2 + gt] = 0u;
                if (gt < S) { sj[gt] = 0; sjend[gt] = 0; spar[gt] = -1; }
                while (true) {
                    grp.sync();
                    // slot refill: thread c < S advances its chain or takes the next parent
                    if (gt < 64) {
                        const int c = gt;
                        bool fresh = false, act = false;
                        if (c < S) {
                            if ((m32[2 + (c >> 5)] >> (c & 31)) & 1u) sj[c] += 1;
                            if (sj[c] >= sjend[c]) {
                                const int qi = atomicAdd(&gint[0], 1);
                                if (qi < nq) {
                                    const int k = keys[qi] & 0xffff;
                                    spar[c] = k;
                                    sj[c] = ids[k];
                                    sjend[c] = ids[k] + cnt[k];
                                    fresh = true;
                                    sL[c] = Lc[k];
                                    sP[c] = Pc[k];
                                    spost[c] = gamma * Lc[k] + Pc[k];
                                }
                            }
                            act = sj[c] < sjend[c];
                            sdt[c] = act ? dtau[sj[c]] : 0.0;
                        }
                        const unsigned fm = __ballot_sync(FULL, fresh), am = __ballot_sync(FULL, act);
                        if (lane == 0) { m32[0 + wl] = fm; m32[2 + wl] = am; m32[4 + wl] = 0u; }
                    }
                    grp.sync();
                    const unsigned long long actm = masks[1], frm = masks[0];
                    if (actm == 0ull) break;
                    // chain start: parent state of fresh slots (coalesced over
                    // dimensions), momentum draws and their kinetic energy
                    if (frm != 0ull)
                        for (int e = gt; e < S * DP; e += NTH) {
                            const int c = e / DP, r = e % DP;
                            if ((frm >> c) & 1ull) tXC[r * TS + c] = r < D ? f32_of_f32valued(parts[(size_t)spar[c] * D + r]) : 0.0f;
                        }
                    float kin = 0.0f;
                    {
                        // dimensions in pairs: one Philox block gives both normals
                        const bool on = (actm >> cs) & 1ull;
                        const int jj = sj[cs];
                        for (int r0 = 2 * part; r0 < DP; r0 += 2 * NPART) {
                            float p0 = 0.0f, p1 = 0.0f;
                            if (on && r0 < D) {
                                const float2 z = rng_normal2_f(a.seed, stream, P_MOM, iter, jj, (uint64_t)(r0 >> 1));
                                p0 = z.x * (float)tisc[r0];
                                kin += p0 * (float)tcov[r0] * p0 * 0.5f;
                                if (r0 + 1 < D) {
                                    p1 = z.y * (float)tisc[r0 + 1];
                                    kin += p1 * (float)tcov[r0 + 1] * p1 * 0.5f;
                                }
                            }
                            tP[r0 * TS + cs] = p0;
                            tP[(r0 + 1) * TS + cs] = p1;
                        }
                    }
                    grp.sync();
#pragma unroll
                    for (int bb = 0; bb < NTW; ++bb) {
                        const int c0 = 8 * (nt0 + bb) + 2 * t4;
                        dts[bb][0] = (float)sdt[c0];
                        dts[bb][1] = (float)sdt[c0 + 1];
                    }
                    // Entries of idle slots and of rows beyond D start at x = p = 0 and
                    // idle slots have step size 0 (sdt), so the step below leaves them
                    // unchanged without a per-entry select: the rows beyond D have zero
                    // gradient (M, c and the stage mean are 0 there), and an idle slot's
                    // momentum and position updates are multiplied by its zero step size.
                    float cdt[MTW][NTW][4];
#pragma unroll
                    for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                        for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const int r = 16 * (mt0 + aa) + g + 8 * (e >> 1), c = 8 * (nt0 + bb) + 2 * t4 + (e & 1);
                                const bool on = live_l[aa][e >> 1] && ((actm >> c) & 1ull);
                                cdt[aa][bb][e] = cov_l[aa][e >> 1] * dts[bb][e & 1];
                                x[aa][bb][e] = on ? tXC[r * TS + c] : 0.0f;
                                p[aa][bb][e] = on ? tP[r * TS + c] : 0.0f;
                            }
                    write_b(0);
                    // leapfrog (smc_slip.f90:755-904): P/2 (X P)^ntau X/2
                    int flag = 0;
                    unsigned frozen = 0u;   // this thread's entries of chains that blew up
                    for (int it = 0; it <= a.ntau; ++it) {
                        grp.sync();
                        const unsigned long long blm = masks[2];
                        const __nv_bfloat16 *bh = (const __nv_bfloat16 *)(Bhi + 2 * (size_t)(it & 1) * L_::B_BYTES);
                        const __nv_bfloat16 *bl = (const __nv_bfloat16 *)(Bhi + (2 * (size_t)(it & 1) + 1) * L_::B_BYTES);
                        // all B fragments first (the loads pipeline), then three
                        // independent accumulation chains: lo*hi, hi*lo, hi*hi
                        float acc[MTW][NTW][4], acc1[MTW][NTW][4], acc2[MTW][NTW][4];
#pragma unroll
                        for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                            for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                                for (int e = 0; e < 4; ++e) acc[aa][bb][e] = acc1[aa][bb][e] = acc2[aa][bb][e] = 0.0f;
                        constexpr int KTB = (NTW * KT <= 8) ? KT : 1;   // k-tiles of B fragments held at once
                        if constexpr (L_::AGL) {
#pragma unroll
                            for (int kt = 0; kt < RING - 1; ++kt) issue_a(kt);
                        }
#pragma unroll
                        for (int k0 = 0; k0 < KT; k0 += KTB) {
                            uint32_t fbh[KTB][NTW][2], fbl[KTB][NTW][2];
#pragma unroll
                            for (int kk = 0; kk < KTB; ++kk)
#pragma unroll
                                for (int bb = 0; bb < NTW; ++bb) {
                                    const int krow = 16 * (k0 + kk) + (lane & 7) + 8 * ((lane >> 3) & 1);
                                    const int ncol = 8 * (nt0 + bb);
                                    ldsm_x2_t(fbh[kk][bb], bh + krow * BST + ncol);
                                    ldsm_x2_t(fbl[kk][bb], bl + krow * BST + ncol);
                                }
#pragma unroll
                            for (int kk = 0; kk < KTB; ++kk) {
                                const int kt = k0 + kk;
                                if constexpr (L_::AGL) {
                                    // groups committed so far: k-tiles 0 .. kt + RING - 1;
                                    // at most RING - 1 pending means k-tile kt has landed
                                    issue_a(kt + RING - 1);
                                    cp_async_wait<RING - 1>();
#pragma unroll
                                    for (int aa = 0; aa < MTW; ++aa) {
                                        const uint4 *rs = wring + (size_t)(2 * ((kt % RING) * MTW + aa)) * 32 + lane;
                                        const uint4 h = rs[0], l = rs[32];
                                        fah[aa][0][0] = h.x; fah[aa][0][1] = h.y; fah[aa][0][2] = h.z; fah[aa][0][3] = h.w;
                                        fal[aa][0][0] = l.x; fal[aa][0][1] = l.y; fal[aa][0][2] = l.z; fal[aa][0][3] = l.w;
                                    }
                                } else if constexpr (!AREG) load_a(kt, 0);
                                const int ks = AREG ? kt : 0;
#pragma unroll
                                for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                                    for (int bb = 0; bb < NTW; ++bb) {
                                        mma16816(acc1[aa][bb], fal[aa][ks], fbh[kk][bb]);
                                        mma16816(acc2[aa][bb], fah[aa][ks], fbl[kk][bb]);
                                        mma16816(acc[aa][bb], fah[aa][ks], fbh[kk][bb]);
                                    }
                            }
                        }
#pragma unroll
                        for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                            for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                                for (int e = 0; e < 4; ++e) acc[aa][bb][e] += acc1[aa][bb][e] + acc2[aa][bb][e];
                        // momentum and position updates with the step factors of this
                        // step; the reflection / blow-up path only for entries that left
                        // [0, max_slip]; chains that blew up stay frozen: their step
                        // size becomes 0 from the step after (rare, warp-uniform branch)
                        if (blm != 0ull) {
#pragma unroll
                            for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                                for (int j = 0; j < 2; ++j)
                                    if ((blm >> (8 * (nt0 + bb) + 2 * t4 + j)) & 1ull) {
                                        dts[bb][j] = 0.0f;
#pragma unroll
                                        for (int aa = 0; aa < MTW; ++aa) {
                                            cdt[aa][bb][j] = 0.0f;
                                            cdt[aa][bb][2 + j] = 0.0f;
                                            frozen |= (1u << ((aa * NTW + bb) * 4 + j)) | (1u << ((aa * NTW + bb) * 4 + 2 + j));
                                        }
                                    }
                        }
                        const float hs = it == 0 ? 0.5f : 1.0f, xs = it == a.ntau ? 0.5f : 1.0f;
                        // common step: update and one range test; entries that left the
                        // box (reflection, or |x| > 1e3: the chain blows up) go through a
                        // warp-uniform branch
                        unsigned outmask = 0u;
#pragma unroll
                        for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                            for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    const int h = e >> 1;
                                    const float gr = cv_l[aa][h] + acc[aa][bb][e];
                                    const float pn = p[aa][bb][e] - gr * (hs * dts[bb][e & 1]);
                                    const float xn = x[aa][bb][e] + cdt[aa][bb][e] * xs * pn;
                                    x[aa][bb][e] = xn;
                                    p[aa][bb][e] = pn;
                                    const bool out = !(xn >= 0.0f && xn <= mx);
                                    outmask |= out ? 1u << ((aa * NTW + bb) * 4 + e) : 0u;
                                }
                        outmask &= ~frozen;   // a blown chain keeps its last state
                        if (__any_sync(FULL, outmask != 0u)) {
#pragma unroll
                            for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                                for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                                    for (int e = 0; e < 4; ++e) {
                                        if (!((outmask >> ((aa * NTW + bb) * 4 + e)) & 1u)) continue;
                                        const int c = 8 * (nt0 + bb) + 2 * t4 + (e & 1);
                                        float &xe = x[aa][bb][e];
                                        if ((xe < 0.0f ? -xe : xe) > 1e3f) atomicOr(&masks[2], 1ull << c);
                                        else reflect_fold(xe, p[aa][bb][e], mx, imx);
                                    }
                        }
                        if (it < a.ntau) {
                            write_b((it + 1) & 1);
                        } else {
                            // end state into the slot-layout tiles; offsets into the idle B buffer
                            float *dl = (float *)(Bhi + 2 * (size_t)((it + 1) & 1) * L_::B_BYTES);
#pragma unroll
                            for (int aa = 0; aa < MTW; ++aa)
#pragma unroll
                                for (int bb = 0; bb < NTW; ++bb)
#pragma unroll
                                    for (int e = 0; e < 4; ++e) {
                                        const int h = e >> 1;
                                        const int r = 16 * (mt0 + aa) + g + 8 * h, c = 8 * (nt0 + bb) + 2 * t4 + (e & 1);
                                        tX[r * TS + c] = x[aa][bb][e];
                                        tP[r * TS + c] = p[aa][bb][e];
                                        dl[r * TS + c] = live_l[aa][h] ? x[aa][bb][e] - mean_l[aa][h] : 0.0f;
                                    }
                        }
                    }
                    status |= flag;
                    grp.sync();
                    // end point in the slot layout: likelihood and prior offsets,
                    // kinetic energy, tuning distance (partial over this thread's dimensions)
                    const unsigned long long blm = masks[2];
                    const float *dl = (const float *)(Bhi + 2 * (size_t)((a.ntau + 1) & 1) * L_::B_BYTES);
                    // FP32 per-thread partial sums: the expansion point (the stage
                    // mean) is FP32-exact, so these are offsets from L(sbar), P(sbar)
                    float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f, q3 = 0.0f;
                    const bool slot_on = (actm >> cs) & 1ull;
                    // rows part + i NPART of A times the offsets: RPT independent chains
                    constexpr int RPT = DP / NPART;
                    float af[RPT];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) af[i] = 0.0f;
                    if constexpr (L_::AGL) {
                        // the FP32 Gram matrix from global memory, KC columns at a time
                        // staged through the A ring (idle: no copy is in flight here)
                        float *As = (float *)aring;
                        constexpr int KC = (int)(L_::ring_bytes(WG) / (DP * sizeof(float)));
                        for (int k0 = 0; k0 < D; k0 += KC) {
                            const int kn = min(KC, D - k0);
                            grp.sync();
                            for (int e = gt; e < kn * DP; e += NTH) {
                                const int kk = e / DP, r = e % DP;
                                As[e] = r < D ? A32[(size_t)(k0 + kk) * D + r] : 0.0f;
                            }
                            grp.sync();
                            if (slot_on)
                                for (int kk = 0; kk < kn; ++kk) {
                                    const float dk = dl[(k0 + kk) * TS + cs];
                                    const float *ak = As + kk * DP + part;
#pragma unroll
                                    for (int i = 0; i < RPT; ++i) af[i] = fmaf(ak[i * NPART], dk, af[i]);
                                }
                        }
                    } else if (slot_on) {
                        if constexpr (L_::A32_GLOBAL) {
                            // MMAQ: the FP32 Gram matrix from global memory (column-major,
                            // leading dimension D; L1/L2-resident), rows >= D skipped
                            const float *Ag = A32 + part;
                            bool rl[RPT];
#pragma unroll
                            for (int i = 0; i < RPT; ++i) rl[i] = part + i * NPART < D;
#pragma unroll 4
                            for (int k = 0; k < D; ++k) {
                                const float dk = dl[k * TS + cs];
                                const float *ak = Ag + (size_t)k * D;
#pragma unroll
                                for (int i = 0; i < RPT; ++i)
                                    if (rl[i]) af[i] = fmaf(ak[i * NPART], dk, af[i]);
                            }
                        } else {
                            for (int k = 0; k < D; ++k) {
                                const float dk = dl[k * TS + cs];
                                const float *ak = tA32 + k * DP + part;
#pragma unroll
                                for (int i = 0; i < RPT; ++i) af[i] = fmaf(ak[i * NPART], dk, af[i]);
                            }
                        }
                    }
                    if (slot_on) {
#pragma unroll
                        for (int i = 0; i < RPT; ++i) {
                            const int r = part + i * NPART;
                            if (r >= D) continue;
                            const float dr = dl[r * TS + cs];
                            q0 += (float)tvg[r] * dr + 0.5f * dr * af[i];
                            q1 += (float)tvh[r] * dr;
                            const float pr = tP[r * TS + cs];
                            q2 += 0.5f * pr * (float)tcov[r] * pr;
                            const float dx = tX[r * TS + cs] - tXC[r * TS + cs];
                            q3 += dx * dx * (float)ticov[r];
                        }
                        const float i2a = (float)(1.0 / (2.0 * alpha2));
                        for (int r2 = part; r2 < m.nrow; r2 += NPART) {
                            float tt = 0.0f;
#pragma unroll
                            for (int k9 = 0; k9 < 9; ++k9) {
                                const int cl = __ldg(m.l_col + r2 * 9 + k9);
                                if (cl >= 0) tt = fmaf(__ldg(lv32 + r2 * 9 + k9), dl[cl * TS + cs], tt);
                            }
                            q1 += tt * tt * i2a;
                        }
                    }
                    float *redf = (float *)red;
                    redf[0 * NTH + part * S + cs] = q0;
                    redf[1 * NTH + part * S + cs] = q1;
                    redf[2 * NTH + part * S + cs] = q2;
                    redf[3 * NTH + part * S + cs] = q3;
                    redf[4 * NTH + part * S + cs] = kin;
                    grp.sync();
                    // Metropolis test and bookkeeping (smc_slip.f90:695-716, 1057-1094)
                    if (gt < 64) {
                        const int c = gt;
                        bool accd = false;
                        if (c < S && ((actm >> c) & 1ull)) {
                            const float *redf = (const float *)red;
                            float q5[5];
#pragma unroll
                            for (int q = 0; q < 5; ++q) {
                                float tt = 0.0f;
                                for (int pt = 0; pt < NPART; ++pt) tt += redf[q * NTH + pt * S + c];
                                q5[q] = tt;
                            }
                            const int jj = sj[c];
                            const bool blown = (blm >> c) & 1ull;
                            const double Lx = (double)q5[0] + Lbar, Px = (double)q5[1] + Pbar;
                            const double post = gamma * Lx + Px;
                            const double ham = blown ? 1e20 : post + (double)q5[2];
                            const double dham = (spost[c] + (double)q5[4]) - ham;
                            const float dhf = (float)fmax(dham, -1e30);
                            if (tuning) score[jj] = blown ? 0.0 : (double)(q5[3] * expf(fminf(0.0f, dhf)));
                            const double u = rng_uniform(a.seed, stream, P_MH, iter, jj, 0);
                            if (!blown && dhf > logf((float)u)) {
                                accd = true;
                                sL[c] = Lx;
                                sP[c] = Px;
                                spost[c] = post;
                            }
                            if (!tuning) {
                                Ln[jj] = sL[c];
                                Pn[jj] = sP[c];
                            }
                        }
                        const unsigned am = __ballot_sync(FULL, accd);
                        if (lane == 0) m32[6 + wl] = am;
                    }
                    grp.sync();
                    const unsigned long long accm = masks[3];
                    if ((accm >> cs) & 1ull)
                        for (int r = part; r < DP; r += NPART) tXC[r * TS + cs] = tX[r * TS + cs];
                    grp.sync();
                    if (!tuning)
                        for (int e = gt; e < S * DP; e += NTH) {
                            const int c = e / DP, r = e % DP;
                            if (r < D && ((actm >> c) & 1ull)) pnew[(size_t)sj[c] * D + r] = (double)tXC[r * TS + c];
                        }
                }
                grp.sync();
            } else if constexpr (ENG == ENG_GL) {
                // ================= global-matrix engine (any D up to DP): S = 16
                // slots per group of WG warps.  The stage matrix M (D x D,
                // column-major, T) is in global memory and each step streams it
                // once; the slots' operand (MIXED: offsets x - sbar; FP64: x) is a
                // [row][slot] tile in shared memory.  Thread (sg, t') owns slots
                // sg * SPT .. + SPT - 1 and rows t', t' + RP, ... (R rows): its
                // positions and momenta stay in registers for the trajectory.
                // Chain states (the last accepted positions) are kept per slot
                // in global memory (InnerArgs::glxc).
                constexpr int S = L_::S, SPT = L_::GL_SPT, SG = S / SPT, NTH = 32 * WG, RP = NTH / SG;
                constexpr int R = DP / RP, WPG = RP / 32;   // rows per thread, warps per slot group
                static_assert(R * RP == DP && SG * SPT == S && S <= 32, "global-matrix engine tiling");
                const int sg = gt / RP, row0 = gt % RP, s0 = sg * SPT;
                T *Xs = Xw0;
                unsigned *m32 = (unsigned *)masks;   // [0] fresh [2] active [4] blown [6] accepted
                const T *Mg = (const T *)a.mgl + (size_t)th * D * D;
                T *xct = (T *)a.glxc + (size_t)th * S * D;
                T cov_r[R], mean_r[R], cv_r[R], isc_r[R];
                double vcov_r[R];
                bool live_r[R];
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    const int r = row0 + i * RP;
                    live_r[i] = r < D;
                    cov_r[i] = tcov[r];
                    mean_r[i] = tmean[r];
                    cv_r[i] = tcv[r];
                    isc_r[i] = tisc[r];
                    vcov_r[i] = vcov[r];
                }
                double *redd = red;   // [q][warp][slot in group]
                if (gt == 0) gint[0] = 0;
                if (gt < 8) m32[gt] = 0u;
                if (gt < S) { sj[gt] = 0; sjend[gt] = 0; spar[gt] = -1; }
                // operand tile from the thread's rows (MIXED: offsets from the stage mean)
                auto write_x = [&](const T (&xx)[R][SPT], unsigned actm) {
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        const int r = row0 + i * RP;
                        T v[SPT];
#pragma unroll
                        for (int q = 0; q < SPT; ++q) {
                            const bool on = live_r[i] && ((actm >> (s0 + q)) & 1u);
                            v[q] = on ? (MIXED ? xx[i][q] - mean_r[i] : xx[i][q]) : T(0);
                        }
                        if constexpr (sizeof(T) == 4) {
#pragma unroll
                            for (int q = 0; q < SPT; q += 4)
                                *reinterpret_cast<float4 *>(Xs + r * S + s0 + q) =
                                    make_float4((float)v[q], (float)v[q + 1], (float)v[q + 2], (float)v[q + 3]);
                        } else {
#pragma unroll
                            for (int q = 0; q < SPT; q += 2)
                                *reinterpret_cast<double2 *>(Xs + r * S + s0 + q) = make_double2(v[q], v[q + 1]);
                        }
                    }
                };
                while (true) {
                    grp.sync();
                    // slot refill: thread c < S advances its chain or takes the next parent
                    if (gt < 32) {
                        const int c = gt;
                        bool fresh = false, act = false;
                        if (c < S) {
                            if ((m32[2] >> c) & 1u) sj[c] += 1;
                            if (sj[c] >= sjend[c]) {
                                const int qi = atomicAdd(&gint[0], 1);
                                if (qi < nq) {
                                    const int k = keys[qi] & 0xffff;
                                    spar[c] = k;
                                    sj[c] = ids[k];
                                    sjend[c] = ids[k] + cnt[k];
                                    fresh = true;
                                    sL[c] = Lc[k];
                                    sP[c] = Pc[k];
                                    spost[c] = gamma * Lc[k] + Pc[k];
                                }
                            }
                            act = sj[c] < sjend[c];
                            sdt[c] = act ? dtau[sj[c]] : 0.0;
                        }
                        const unsigned fm = __ballot_sync(FULL, fresh), am = __ballot_sync(FULL, act);
                        if (lane == 0) { m32[0] = fm; m32[2] = am; m32[4] = 0u; }
                    }
                    grp.sync();
                    const unsigned actm = m32[2], frm = m32[0];
                    if (actm == 0u) break;
                    // chain start: a fresh slot's chain state is its parent
                    if (frm != 0u) {
                        for (int e = gt; e < S * D; e += NTH) {
                            const int c = e / D, r = e % D;
                            if ((frm >> c) & 1u) xct[e] = (T)parts[(size_t)spar[c] * D + r];
                        }
                        grp.sync();
                    }
                    // per-slot sums over the thread's rows, reduced over each warp into
                    // redd[q][warp][slot]: q = 0 likelihood, 1 prior, 2 end kinetic
                    // energy, 3 tuning distance, 4 start kinetic energy
                    auto put = [&](double (&v)[SPT], int qq) {
                        const double t = wreduce_n<SPT>(v, lane);
                        if ((lane % (32 / SPT)) == 0) redd[(qq * WG + wl) * SPT + lane / (32 / SPT)] = t;
                    };
                    T x[R][SPT], p[R][SPT], dts[SPT];
                    double kin[SPT];
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        const int c = s0 + q;
                        const bool on = (actm >> c) & 1u;
                        const int jj = sj[c];
                        dts[q] = (T)sdt[c];
                        kin[q] = 0.0;
#pragma unroll
                        for (int i = 0; i < R; ++i) {
                            const int r = row0 + i * RP;
                            T xv = T(0), pv = T(0);
                            if (on && live_r[i]) {
                                xv = xct[(size_t)c * D + r];
                                if constexpr (MIXED) {
                                    const float2 z = rng_normal2_f(a.seed, stream, P_MOM, iter, jj, (uint64_t)(r >> 1));
                                    pv = ((r & 1) ? z.y : z.x) * isc_r[i];
                                    kin[q] += (double)(pv * cov_r[i] * pv * 0.5f);
                                } else {
                                    pv = (T)(rng_normal(a.seed, stream, P_MOM, iter, jj, r) / sqrt(vcov_r[i]));
                                    kin[q] += (double)pv * vcov_r[i] * (double)pv / 2.0;
                                }
                            }
                            x[i][q] = xv;
                            p[i][q] = pv;
                        }
                    }
                    put(kin, 4);
                    // leapfrog (smc_slip.f90:755-904): P/2 (X P)^ntau X/2
                    int flag = 0;
                    const float imx = 1.0f / (float)mx;
                    for (int it = 0; it <= a.ntau; ++it) {
                        write_x(x, actm);
                        grp.sync();
                        T acc[R][SPT];
                        gl_gemm<T, R, SPT, RP, S, L_::GL_RING, NTH>(Mg, D, Xs, row0, s0, Xw1, gt, acc);
                        grp.sync();
                        const unsigned blm = m32[4];
                        const T hs = it == 0 ? T(0.5) : T(1), xs = it == a.ntau ? T(0.5) : T(1);
#pragma unroll
                        for (int q = 0; q < SPT; ++q) {
                            const int c = s0 + q;
                            const bool on = ((actm >> c) & 1u) && !((blm >> c) & 1u);
#pragma unroll
                            for (int i = 0; i < R; ++i) {
                                if (!(on && live_r[i])) continue;
                                const T gr = MIXED ? cv_r[i] + acc[i][q] : acc[i][q] - cv_r[i];
                                p[i][q] = p[i][q] - gr * hs * dts[q];
                                x[i][q] = x[i][q] + cov_r[i] * p[i][q] * xs * dts[q];
                                if constexpr (MIXED) {
                                    const bool blow = (x[i][q] < T(0) ? -x[i][q] : x[i][q]) > T(1e3);
                                    if (blow) atomicOr(&m32[4], 1u << c);
                                    else reflect_fold(x[i][q], p[i][q], mx, imx);
                                } else if (blow_or_reflect<T>(x[i][q], p[i][q], mx, flag)) {
                                    atomicOr(&m32[4], 1u << c);
                                }
                            }
                        }
                    }
                    status |= flag;
                    // end point: the operand (offsets, or positions in FP64) and A times it
                    write_x(x, actm);
                    grp.sync();
                    const unsigned blm = m32[4];
                    T af[R][SPT];
                    if constexpr (MIXED) gl_gemm<T, R, SPT, RP, S, L_::GL_RING, NTH>((const T *)A32, D, Xs, row0, s0, Xw1, gt, af);
                    else gl_gemm<T, R, SPT, RP, S, L_::GL_RING, NTH>((const T *)Ath, D, Xs, row0, s0, Xw1, gt, af);
                    // per-slot sums over the thread's rows, one quantity at a time
                    double v[SPT];
                    // likelihood term (MIXED: g.delta + delta.A delta / 2; FP64: x.A x - 2 b.x)
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        v[q] = 0.0;
                        if (!((actm >> (s0 + q)) & 1u)) continue;
#pragma unroll
                        for (int i = 0; i < R; ++i) {
                            if (!live_r[i]) continue;
                            const int r = row0 + i * RP;
                            if constexpr (MIXED) {
                                const float dr = x[i][q] - mean_r[i];
                                v[q] += (double)((float)tvg[r] * dr + 0.5f * dr * af[i][q]);
                            } else {
                                const double xv = (double)x[i][q];
                                v[q] += xv * (double)af[i][q] - 2.0 * vb[r] * xv;
                            }
                        }
                    }
                    put(v, 0);
                    // prior term (MIXED: h.delta + |L delta|^2 / (2 alpha^2); FP64: |L x|^2 / (2 alpha^2))
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        v[q] = 0.0;
                        if constexpr (MIXED) {
                            if (!((actm >> (s0 + q)) & 1u)) continue;
#pragma unroll
                            for (int i = 0; i < R; ++i)
                                if (live_r[i]) v[q] += (double)((float)tvh[row0 + i * RP] * (x[i][q] - mean_r[i]));
                        }
                    }
                    for (int r2 = row0; r2 < m.nrow; r2 += RP) {
#pragma unroll
                        for (int q = 0; q < SPT; ++q) {
                            const int c = s0 + q;
                            if (!((actm >> c) & 1u)) continue;
                            double t = 0.0;
                            for (int k9 = 0; k9 < 9; ++k9) {
                                const int cl = m.l_col[r2 * 9 + k9];
                                if (cl >= 0) t += lv[(size_t)r2 * 9 + k9] * (double)Xs[cl * S + c];
                            }
                            v[q] += t * t / (2.0 * alpha2);
                        }
                    }
                    put(v, 1);
                    // end kinetic energy
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        v[q] = 0.0;
                        if (!((actm >> (s0 + q)) & 1u)) continue;
#pragma unroll
                        for (int i = 0; i < R; ++i) {
                            if (!live_r[i]) continue;
                            if constexpr (MIXED) v[q] += (double)(0.5f * p[i][q] * cov_r[i] * p[i][q]);
                            else v[q] += (double)p[i][q] * vcov_r[i] * (double)p[i][q] / 2.0;
                        }
                    }
                    put(v, 2);
                    // tuning distance from the chain start
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        v[q] = 0.0;
                        const int c = s0 + q;
                        if (!((actm >> c) & 1u)) continue;
#pragma unroll
                        for (int i = 0; i < R; ++i) {
                            if (!live_r[i]) continue;
                            const int r = row0 + i * RP;
                            const T xcv = xct[(size_t)c * D + r];
                            if constexpr (MIXED) {
                                const float dx = x[i][q] - xcv;
                                v[q] += (double)(dx * dx * (float)ticov[r]);
                            } else {
                                const double dx = (double)x[i][q] - (double)xcv;
                                v[q] += dx * dx / vcov_r[i];
                            }
                        }
                    }
                    put(v, 3);
                    grp.sync();
                    // Metropolis test and bookkeeping (smc_slip.f90:695-716, 1057-1094)
                    if (gt < 32) {
                        const int c = gt;
                        bool accd = false;
                        if (c < S && ((actm >> c) & 1u)) {
                            const int g0 = (c / SPT) * WPG, cq = c % SPT;
                            double q5[5];
#pragma unroll
                            for (int qq = 0; qq < 5; ++qq) {
                                double t = 0.0;
                                for (int w2 = 0; w2 < WPG; ++w2) t += redd[(qq * WG + g0 + w2) * SPT + cq];
                                q5[qq] = t;
                            }
                            const int jj = sj[c];
                            const bool blown = (blm >> c) & 1u;
                            const double Lx = MIXED ? q5[0] + Lbar : (q5[0] + dsd) / 2.0 + lconst;
                            const double Px = MIXED ? q5[1] + Pbar : q5[1];
                            const double post = gamma * Lx + Px;
                            const double ham = blown ? 1e20 : post + q5[2];
                            const double dham = (spost[c] + q5[4]) - ham;
                            if (tuning) score[jj] = blown ? 0.0 : q5[3] * exp(fmin(0.0, dham));
                            const double u = rng_uniform(a.seed, stream, P_MH, iter, jj, 0);
                            if (!blown && dham > log(u)) {
                                accd = true;
                                sL[c] = Lx;
                                sP[c] = Px;
                                spost[c] = post;
                            }
                            if (!tuning) {
                                Ln[jj] = sL[c];
                                Pn[jj] = sP[c];
                            }
                        }
                        const unsigned am = __ballot_sync(FULL, accd);
                        if (lane == 0) m32[6] = am;
                    }
                    grp.sync();
                    const unsigned accm = m32[6];
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        const int c = s0 + q;
                        if (!((actm >> c) & 1u)) continue;
                        const bool accd = (accm >> c) & 1u;
#pragma unroll
                        for (int i = 0; i < R; ++i) {
                            if (!live_r[i]) continue;
                            const int r = row0 + i * RP;
                            T *xp = xct + (size_t)c * D + r;
                            if (accd) *xp = x[i][q];
                            if (!tuning) pnew[(size_t)sj[c] * D + r] = (double)(accd ? x[i][q] : *xp);
                        }
                    }
                }
                grp.sync();
            } else if constexpr (TC) {
                // ================= tcgen05 engine: S slots per group, thread
                // (row t) owns dimension r = t % DP of slots s0 .. s0+15
                constexpr int S = L_::S, SPT = 16;
                const int r = gt % DP, s0 = (gt / DP) * SPT;
                const bool rowlive = r < D;
                const float cov_r = (float)tcov[r], mean_r = (float)tmean[r], cv_r = (float)tcv[r];
                const float isc_r = (float)tisc[r];
                const double vcov_r = vcov[r], vmean_r = vmean[r], vg_r = vg[r], vh_r = vh[r];
                const uint32_t tcol = tmem_base + (uint32_t)(grp.id * S);
                const uint32_t taddr = tcol + ((uint32_t)(32 * wl) << 16) + (uint32_t)s0;
                const uint32_t idesc = tc::idesc_bf16_f32(128, S);
                const uint32_t sa_hi = tc::smem_u32(Ahi), sa_lo = tc::smem_u32(Alo);
                const uint32_t sb_hi = tc::smem_u32(Bhi), sb_lo = tc::smem_u32(Blo);
                unsigned *m32 = (unsigned *)masks;   // halves: [0,1] fresh [2,3] active [4,5] blown [6,7] accepted
                float xc[SPT], x[SPT], p[SPT], kin[SPT], dts[SPT];
#pragma unroll
                for (int s = 0; s < SPT; ++s) xc[s] = 0.0f;
                if (gt == 0) gint[0] = 0;
                if (gt < 2) m32[2 + gt] = 0u;
                if (gt < S) { sj[gt] = 0; sjend[gt] = 0; spar[gt] = -1; }
                bool failed = false;
                while (true) {
                    grp.sync();
                    // slot refill: thread c < S advances its chain or takes the next parent
                    if (gt < 64) {
                        const int c = gt;
                        bool fresh = false, act = false;
                        if (c < S) {
                            if ((m32[2 + (c >> 5)] >> (c & 31)) & 1u) sj[c] += 1;
                            if (sj[c] >= sjend[c]) {
                                const int qi = atomicAdd(&gint[0], 1);
                                if (qi < nq) {
                                    const int k = keys[qi] & 0xffff;
                                    spar[c] = k;
                                    sj[c] = ids[k];
                                    sjend[c] = ids[k] + cnt[k];
                                    fresh = true;
                                    sL[c] = Lc[k];
                                    sP[c] = Pc[k];
                                    spost[c] = gamma * Lc[k] + Pc[k];
                                }
                            }
                            act = sj[c] < sjend[c];
                            sdt[c] = act ? dtau[sj[c]] : 0.0;
                        }
                        const unsigned fm = __ballot_sync(FULL, fresh), am = __ballot_sync(FULL, act);
                        if (lane == 0) { m32[0 + wl] = fm; m32[2 + wl] = am; m32[4 + wl] = 0u; }
                    }
                    grp.sync();
                    const unsigned long long actm = masks[1], frm = masks[0];
                    if (actm == 0ull) break;
                    // chain start: parent state, momentum draw, first operand tile
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        const int c = s0 + s;
                        const bool on = rowlive && ((actm >> c) & 1ull);
                        if ((frm >> c) & 1ull) xc[s] = on ? (float)parts[(size_t)spar[c] * D + r] : 0.0f;
                        dts[s] = (float)sdt[c];
                        float pv = 0.0f;
                        if (on) pv = rng_normal_f(a.seed, stream, P_MOM, iter, sj[c], r) * isc_r;
                        kin[s] = pv * cov_r * pv * 0.5f;
                        p[s] = pv;
                        x[s] = xc[s];
                        __nv_bfloat16 hi, lo;
                        tc::split_bf16(rowlive ? x[s] - mean_r : 0.0f, hi, lo);
                        const uint32_t off = tc::core_offset(c, r, L_::LBO_B);
                        *(__nv_bfloat16 *)(Bhi + off) = hi;
                        *(__nv_bfloat16 *)(Blo + off) = lo;
                    }
                    // leapfrog (smc_slip.f90:755-904): P/2 (X P)^ntau X/2
                    int flag = 0;
                    for (int it = 0; it <= a.ntau; ++it) {
                        tc::fence_async_smem();
                        tc::fence_before_sync();
                        grp.sync();
                        if (gint[3]) { failed = true; break; }
                        const unsigned long long blm = masks[2];
                        if (gt == 0) {
                            tc::fence_after_sync();
#pragma unroll
                            for (int kk = 0; kk < DP / 16; ++kk) {
                                const uint64_t ah = tc::smem_desc(sa_hi + kk * 2 * L_::LBO_A, L_::LBO_A, 128);
                                const uint64_t al = tc::smem_desc(sa_lo + kk * 2 * L_::LBO_A, L_::LBO_A, 128);
                                const uint64_t bh = tc::smem_desc(sb_hi + kk * 2 * L_::LBO_B, L_::LBO_B, 128);
                                const uint64_t bl = tc::smem_desc(sb_lo + kk * 2 * L_::LBO_B, L_::LBO_B, 128);
                                tc::mma_bf16(tcol, ah, bh, idesc, kk > 0 ? 1u : 0u);
                                tc::mma_bf16(tcol, ah, bl, idesc, 1u);
                                tc::mma_bf16(tcol, al, bh, idesc, 1u);
                            }
                            tc::mma_commit(mbar);
                        }
                        if (!tc::mbar_wait(mbar, phase, WAIT_TRIES)) gint[3] = 1;
                        phase ^= 1u;
                        tc::fence_after_sync();
                        float acc[SPT];
                        tc::tmem_ld16(taddr, acc);
                        tc::tmem_wait_ld();
                        const float hstep = it == 0 ? 0.5f : 1.0f, xstep = it == a.ntau ? 0.5f : 1.0f;
#pragma unroll
                        for (int s = 0; s < SPT; ++s) {
                            const int c = s0 + s;
                            if (rowlive && ((actm >> c) & 1ull) && !((blm >> c) & 1ull)) {
                                const float gr = cv_r + acc[s];
                                p[s] = p[s] - gr * hstep * dts[s];
                                x[s] = x[s] + cov_r * p[s] * xstep * dts[s];
                                const bool blow = (x[s] < 0.0f ? -x[s] : x[s]) > 1e3f;
                                if (blow) atomicOr(&masks[2], 1ull << c);
                                else reflect_fold(x[s], p[s], mx, 1.0f / mx);
                            }
                            const float dl = rowlive ? x[s] - mean_r : 0.0f;
                            if (it < a.ntau) {
                                __nv_bfloat16 hi, lo;
                                tc::split_bf16(dl, hi, lo);
                                const uint32_t off = tc::core_offset(c, r, L_::LBO_B);
                                *(__nv_bfloat16 *)(Bhi + off) = hi;
                                *(__nv_bfloat16 *)(Blo + off) = lo;
                            } else {
                                Xf[r * S + c] = dl;
                            }
                        }
                    }
                    status |= flag;
                    if (failed) break;
                    grp.sync();
                    // end point: per-slot sums over dimensions of the likelihood and
                    // prior offsets, kinetic energies and the tuning distance
                    const unsigned long long blm = masks[2];
                    const int wib = r >> 5;
                    double v[SPT];
                    {
                        float af[SPT];
#pragma unroll
                        for (int s = 0; s < SPT; ++s) af[s] = 0.0f;
                        if (rowlive)
                            for (int k = 0; k < D; ++k) {
                                const float ak = A32[(size_t)k * D + r];
                                const float *xk = Xf + k * S + s0;
#pragma unroll
                                for (int s = 0; s < SPT; ++s) af[s] = fmaf(ak, xk[s], af[s]);
                            }
#pragma unroll
                        for (int s = 0; s < SPT; ++s) {
                            const double del = (double)x[s] - vmean_r;
                            v[s] = rowlive ? vg_r * del + 0.5 * (double)Xf[r * S + s0 + s] * (double)af[s] : 0.0;
                        }
                        const double t = wreduce16(v, lane);
                        if (!(lane & 1)) red[0 * 64 + wib * S + s0 + (lane >> 1)] = t;
                    }
                    {
#pragma unroll
                        for (int s = 0; s < SPT; ++s) v[s] = rowlive ? vh_r * ((double)x[s] - vmean_r) : 0.0;
                        for (int r2 = r; r2 < m.nrow; r2 += DP) {
                            double t[SPT];
#pragma unroll
                            for (int s = 0; s < SPT; ++s) t[s] = 0.0;
                            for (int k9 = 0; k9 < 9; ++k9) {
                                const int cl = m.l_col[r2 * 9 + k9];
                                if (cl < 0) continue;
                                const double lvv = lv[(size_t)r2 * 9 + k9];
                                const float *xk = Xf + cl * S + s0;
#pragma unroll
                                for (int s = 0; s < SPT; ++s) t[s] += lvv * (double)xk[s];
                            }
#pragma unroll
                            for (int s = 0; s < SPT; ++s) v[s] += t[s] * t[s] / (2.0 * alpha2);
                        }
                        const double t = wreduce16(v, lane);
                        if (!(lane & 1)) red[1 * 64 + wib * S + s0 + (lane >> 1)] = t;
                    }
                    {
#pragma unroll
                        for (int s = 0; s < SPT; ++s) v[s] = rowlive ? (double)p[s] * vcov_r * (double)p[s] / 2.0 : 0.0;
                        const double t = wreduce16(v, lane);
                        if (!(lane & 1)) red[2 * 64 + wib * S + s0 + (lane >> 1)] = t;
                    }
                    {
#pragma unroll
                        for (int s = 0; s < SPT; ++s) {
                            const double dx = (double)x[s] - (double)xc[s];
                            v[s] = rowlive ? dx * dx / vcov_r : 0.0;
                        }
                        const double t = wreduce16(v, lane);
                        if (!(lane & 1)) red[3 * 64 + wib * S + s0 + (lane >> 1)] = t;
                    }
                    {
#pragma unroll
                        for (int s = 0; s < SPT; ++s) v[s] = (double)kin[s];
                        const double t = wreduce16(v, lane);
                        if (!(lane & 1)) red[4 * 64 + wib * S + s0 + (lane >> 1)] = t;
                    }
                    grp.sync();
                    // Metropolis test and bookkeeping (smc_slip.f90:695-716, 1057-1094)
                    if (gt < 64) {
                        const int c = gt;
                        bool accd = false;
                        if (c < S && ((actm >> c) & 1ull)) {
                            double q5[5];
#pragma unroll
                            for (int q = 0; q < 5; ++q) {
                                double t = 0.0;
                                for (int wb = 0; wb < DP / 32; ++wb) t += red[q * 64 + wb * S + c];
                                q5[q] = t;
                            }
                            const int jj = sj[c];
                            const bool blown = (blm >> c) & 1ull;
                            const double Lx = q5[0] + Lbar, Px = q5[1] + Pbar;
                            const double post = gamma * Lx + Px;
                            const double ham = blown ? 1e20 : post + q5[2];
                            const double dham = (spost[c] + q5[4]) - ham;
                            if (tuning) score[jj] = blown ? 0.0 : q5[3] * exp(fmin(0.0, dham));
                            const double u = rng_uniform(a.seed, stream, P_MH, iter, jj, 0);
                            if (!blown && dham > log(u)) {
                                accd = true;
                                sL[c] = Lx;
                                sP[c] = Px;
                                spost[c] = post;
                            }
                            if (!tuning) {
                                Ln[jj] = sL[c];
                                Pn[jj] = sP[c];
                            }
                        }
                        const unsigned am = __ballot_sync(FULL, accd);
                        if (lane == 0) m32[6 + wl] = am;
                    }
                    grp.sync();
                    const unsigned long long accm = masks[3];
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        const int c = s0 + s;
                        if ((accm >> c) & 1ull) xc[s] = x[s];
                        if (!tuning && rowlive && ((actm >> c) & 1ull)) pnew[(size_t)sj[c] * D + r] = (double)xc[s];
                    }
                }
                grp.sync();
                if (gint[3]) break;
            } else {
                // ================= CUDA-core engine: 8 slots per warp
                if (gt == 0) gint[0] = 0;
                if (lane < CW) { sj[lane] = 0; sjend[lane] = 0; spar[lane] = -1; }
                grp.sync();
                T xc[RT][CTW], x[RT][CTW], p[RT][CTW], acc[RT][CTW];
                const float imxf = 1.0f / (float)mx;
#pragma unroll
                for (int i = 0; i < RT; ++i)
#pragma unroll
                    for (int q = 0; q < CTW; ++q) xc[i][q] = T(0);
                while (true) {
                    // slot refill from the group queue (lane 0), then broadcast
                    if (lane == 0) {
                        for (int c = 0; c < CW; ++c) {
                            sfresh[c] = 0;
                            if (sj[c] >= sjend[c]) {
                                int qi = atomicAdd(&gint[0], 1);
                                if (qi < nq) {
                                    int k = keys[qi] & 0xffff;
                                    spar[c] = k;
                                    sj[c] = ids[k];
                                    sjend[c] = ids[k] + cnt[k];
                                    sfresh[c] = 1;
                                }
                            }
                        }
                    }
                    __syncwarp();
                    bool any = false;
#pragma unroll
                    for (int c = 0; c < CW; ++c) any |= sj[c] < sjend[c];
                    if (!any) break;
                    if (lane < CW) {
                        int c = lane;
                        if (sfresh[c]) {
                            int k = spar[c];
                            sL[c] = Lc[k];
                            sP[c] = Pc[k];
                            spost[c] = gamma * Lc[k] + Pc[k];
                        }
                        sdt[c] = sj[c] < sjend[c] ? dtau[sj[c]] : 0.0;
                        sblown[c] = 0;
                    }
                    __syncwarp();
                    double kin[CTW];
                    T dts[CTW];
                    bool act[CTW];
#pragma unroll
                    for (int q = 0; q < CTW; ++q) {
                        int c = cg * CTW + q;
                        act[q] = sj[c] < sjend[c];
                        dts[q] = (T)sdt[c];
                        kin[q] = 0.0;
                        const int jj = sj[c];
#pragma unroll
                        for (int i = 0; i < RT; ++i) {
                            int r = rg * RT + i;
                            if (sfresh[c]) xc[i][q] = (act[q] && r < D) ? (T)parts[(size_t)spar[c] * D + r] : T(0);
                            T pv = T(0);
                            if (act[q] && r < D) {
                                if (MIXED) {
                                    pv = rng_normal_f(a.seed, stream, P_MOM, iter, jj, r) * tisc[r];
                                    kin[q] += (double)(pv * tcov[r] * pv * T(0.5));
                                } else {
                                    pv = (T)(rng_normal(a.seed, stream, P_MOM, iter, jj, r) / sqrt(vcov[r]));
                                    kin[q] += (double)pv * vcov[r] * (double)pv / 2.0;
                                }
                            }
                            p[i][q] = pv;
                            x[i][q] = xc[i][q];
                            Xw0[r * CW + c] = (r < D) ? (MIXED ? x[i][q] - tmean[r] : x[i][q]) : T(0);
                        }
                        kin[q] = hsum(kin[q]);
                    }
                    if (rg == 0) {
#pragma unroll
                        for (int q = 0; q < CTW; ++q) sham[cg * CTW + q] = spost[cg * CTW + q] + kin[q];
                    }
                    __syncwarp();
                    // leapfrog (smc_slip.f90:755-904): P/2 (X P)^ntau X/2
                    int flag = 0;
                    for (int it = 0; it <= a.ntau; ++it) {
                        T *Xr = (it & 1) ? Xw1 : Xw0;
                        T *Xw = (it & 1) ? Xw0 : Xw1;
                        warp_gemm<T, RT>(Msm, Xr, rg, cg, acc);
                        const T hstep = (it == 0) ? T(0.5) : T(1);
                        const T xstep = (it == a.ntau) ? T(0.5) : T(1);
#pragma unroll
                        for (int q = 0; q < CTW; ++q) {
                            int c = cg * CTW + q;
                            bool live = act[q] && !sblown[c];
#pragma unroll
                            for (int i = 0; i < RT; ++i) {
                                int r = rg * RT + i;
                                if (live && r < D) {
                                    T gr = MIXED ? tcv[r] + acc[i][q] : acc[i][q] - tcv[r];
                                    p[i][q] = p[i][q] - gr * hstep * dts[q];
                                    x[i][q] = x[i][q] + tcov[r] * p[i][q] * xstep * dts[q];
                                    if constexpr (MIXED) {
                                        const bool blow = (x[i][q] < T(0) ? -x[i][q] : x[i][q]) > T(1e3);
                                        if (blow) atomicOr(&sblown[c], 1);
                                        else reflect_fold(x[i][q], p[i][q], mx, imxf);
                                    } else if (blow_or_reflect<T>(x[i][q], p[i][q], mx, flag)) {
                                        atomicOr(&sblown[c], 1);
                                    }
                                }
                                Xw[r * CW + c] = (r < D) ? (MIXED ? x[i][q] - tmean[r] : x[i][q]) : T(0);
                            }
                        }
                        __syncwarp();
                    }
                    status |= flag;
                    // end point: likelihood, prior, kinetic energy, tuning score
                    T *Xf = ((a.ntau + 1) & 1) ? Xw1 : Xw0;
                    double pl[CTW], pk[CTW], psc[CTW], pp[CTW];
#pragma unroll
                    for (int q = 0; q < CTW; ++q) {
                        int c = cg * CTW + q;
                        pl[q] = pk[q] = psc[q] = pp[q] = 0.0;
#pragma unroll
                        for (int i = 0; i < RT; ++i) {
                            int r = rg * RT + i;
                            if (r >= D) continue;
                            double ar = 0.0;
                            if (MIXED) {
                                float af = 0.0f;
                                for (int k = 0; k < D; ++k) af = fmaf(A32[(size_t)k * D + r], (float)Xf[k * CW + c], af);
                                ar = (double)af;
                                double del = (double)x[i][q] - vmean[r];
                                pl[q] += vg[r] * del + 0.5 * (double)Xf[r * CW + c] * ar;
                                pp[q] += vh[r] * del;
                            } else {
                                for (int k = 0; k < D; ++k) ar += Ath[(size_t)k * D + r] * (double)Xf[k * CW + c];
                                double xv = (double)x[i][q];
                                pl[q] += xv * ar - 2.0 * vb[r] * xv;
                            }
                            pk[q] += (double)p[i][q] * vcov[r] * (double)p[i][q] / 2.0;
                            double dx = (double)x[i][q] - (double)xc[i][q];
                            psc[q] += dx * dx / vcov[r];
                        }
                        for (int r = rg; r < m.nrow; r += RGW) {
                            double t = 0.0;
                            for (int k9 = 0; k9 < 9; ++k9) {
                                int cl = m.l_col[r * 9 + k9];
                                if (cl >= 0) t += lv[(size_t)r * 9 + k9] * (double)Xf[cl * CW + c];
                            }
                            pp[q] += t * t / (2.0 * alpha2);
                        }
                        pl[q] = hsum(pl[q]);
                        pk[q] = hsum(pk[q]);
                        psc[q] = hsum(psc[q]);
                        pp[q] = hsum(pp[q]);
                    }
                    // Metropolis test and bookkeeping (smc_slip.f90:695-716, 1057-1094)
                    int accm = 0;
                    if (rg == 0) {
#pragma unroll
                        for (int q = 0; q < CTW; ++q) {
                            int c = cg * CTW + q;
                            if (!act[q]) continue;
                            int jj = sj[c];
                            bool blown = sblown[c];
                            double Lx = MIXED ? pl[q] + Lbar : (pl[q] + dsd) / 2.0 + lconst;
                            double Px = MIXED ? pp[q] + Pbar : pp[q];
                            double post = gamma * Lx + Px;
                            double ham = blown ? 1e20 : post + pk[q];
                            double dham = sham[c] - ham;
                            if (tuning) score[jj] = blown ? 0.0 : psc[q] * exp(fmin(0.0, dham));
                            double u = rng_uniform(a.seed, stream, P_MH, iter, jj, 0);
                            if (!blown && dham > log(u)) {
                                accm |= 1 << q;
                                sL[c] = Lx;
                                sP[c] = Px;
                                spost[c] = post;
                            }
                            if (!tuning) {
                                Ln[jj] = sL[c];
                                Pn[jj] = sP[c];
                            }
                        }
                    }
                    accm = __shfl_sync(FULL, accm, lane & 16);
#pragma unroll
                    for (int q = 0; q < CTW; ++q) {
                        int c = cg * CTW + q;
                        if (!act[q]) continue;
                        bool accd = (accm >> q) & 1;
#pragma unroll
                        for (int i = 0; i < RT; ++i) {
                            int r = rg * RT + i;
                            if (accd) xc[i][q] = x[i][q];
                            if (!tuning && r < D) pnew[(size_t)sj[c] * D + r] = (double)xc[i][q];
                        }
                    }
                    __syncwarp();
                    if (lane < CW && sj[lane] < sjend[lane]) sj[lane] += 1;
                    __syncwarp();
                }
                grp.sync();
            }
            if (tuning) {
                // tuned children in ascending order, then step sizes resampled by score (warp 0)
                for (int q = gt; q < nq; q += gnt) {
                    int k = keys[q] & 0xffff;
                    for (int jj = ids[k]; jj < ids[k] + cnt[k]; ++jj) sub[jj] = 1;
                }
                grp.sync();
                if (wl == 0) {
                    int carry = 0;
                    for (int base = 0; base < N; base += 32) {
                        int jj = base + lane, tot;
                        int v = jj < N ? (sub[jj] == 1) : 0;
                        int ex = wexscan(v, lane, tot);
                        __syncwarp();
                        if (jj < N) {
                            if (v) keys[carry + ex] = jj;
                            sub[jj] = 0;
                        }
                        carry += tot;
                        __syncwarp();
                    }
                    const int msub = carry;
                    double ps2 = 0.0;
                    for (int q = lane; q < msub; q += 32) ps2 += score[keys[q]];
                    double ssum = wsum(ps2);
                    bool degenerate = ssum < 1e-5;
                    if (degenerate) ssum = (double)msub;
                    for (int q = lane; q < msub; q += 32) w[q] = (degenerate ? 1.0 : score[keys[q]]) / ssum;
                    __syncwarp();
                    double uh, ul;
                    rng_quad_uniform(a.seed, stream, RNG_TUNE_RES, iter, uh, ul);
                    long long tot = warp_counts(w, msub, N, uh, ul, sub, lane);
                    __syncwarp();
                    if (tot == N) {
                        int carry2 = 0;
                        for (int base = 0; base < msub; base += 32) {
                            int q = base + lane, tt;
                            int v = q < msub ? sub[q] : 0;
                            int ex = wexscan(v, lane, tt);
                            if (q < msub)
                                for (int r = 0; r < v; ++r) dtn[carry2 + ex + r] = dtau[keys[q]];
                            carry2 += tt;
                        }
                        __syncwarp();
                        for (int k = lane; k < N; k += 32) dtau[k] = dtn[k];
                    } else {
                        status |= SMCGPU_ST_TUNE_COUNT;
                    }
                    __syncwarp();
                    for (int k = lane; k < NP2; k += 32) sub[k] = 0;
                }
                grp.sync();
                dd pd = {0.0, 0.0};
                for (int k = gt; k < N; k += gnt) pd = dd_add_d(pd, dtau[k]);
                dd sm = grp.sum_dd(pd);
                double mean_hi = sm.hi / N;
                double mean_lo = (fma(-mean_hi, (double)N, sm.hi) + sm.lo) / N;
                double lm = log(mean_hi) + mean_lo / mean_hi;
                log_up = lm + log(5.0);
                log_lo = lm - log(5.0);
                grp.sync();
            }
        }
        if (ENG == ENG_TC && gint[3]) {
            // a tensor-core completion wait gave up: abandon this evaluation
            neglog = 1e10;
            status |= SMCGPU_ST_WAIT_CAP;
            break;
        }
        for (size_t e = gt; e < (size_t)N * D; e += gnt) parts[e] = pnew[e];
        for (int k = gt; k < N; k += gnt) { Lc[k] = Ln[k]; Pc[k] = Pn[k]; }
        grp.sync();
        ++iter;
    }
    if constexpr (TC) {
        // an MMA batch whose wait gave up may still be in flight: wait for it
        // (bounded) before the tensor memory is released
        if (gt == 0 && gint[3]) tc::mbar_wait(mbar, phase ^ 1u, WAIT_TRIES);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) status |= __shfl_xor_sync(FULL, status, o);
    if (lane == 0 && status) atomicOr(&gint[2], status);
    grp.sync();
    if (nonfinite) neglog = __longlong_as_double(0x7ff8000000000000LL);   // NaN
    if (gt == 0) {
        int st = gint[2];
        if (!isfinite(neglog)) st |= SMCGPU_ST_NONFINITE;
        a.neglog[th] = neglog;
        atomicOr(a.status + th, st);
        a.nstage[th] = iter - 1;
        if (a.counters) {
            atomicAdd(a.counters, (unsigned long long)(iter - 1));
            atomicAdd(a.counters + 1, (unsigned long long)ntraj);
        }
    }
}

__host__ __device__ constexpr uint32_t tmem_columns(int n) {
    uint32_t c = 32;
    while (c < (uint32_t)n) c <<= 1;
    return c;
}

template <typename T, int RT, int ENG, int WG>
__device__ __forceinline__ void inner_group_entry(const InnerParts &P, int W, int G) {
    extern __shared__ __align__(128) unsigned char smem_all[];
    __shared__ uint32_t tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Group grp;
    grp.id = warp / W;
    grp.W = W;
    grp.wl = warp % W;
    grp.lane = lane;
    grp.gt = grp.wl * 32 + lane;
    grp.nt = 32 * W;
    grp.scr = nullptr;
    uint32_t tmem_base = 0;
    constexpr uint32_t S = Layout<T, RT, ENG>::S;
    const uint32_t ncols = tmem_columns(G * (int)S);
    if constexpr (ENG == ENG_TC) {
        if (warp == 0) {
            tc::tmem_alloc(&tmem_slot, ncols);
            tc::tmem_relinquish();
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        tmem_base = tmem_slot;
    }
    if (grp.id < G) {
        unsigned char *gsm = smem_all + (size_t)grp.id * Layout<T, RT, ENG>::bytes(W);
        const int ntot = P.start[P.n];
        int *queue = P.a[0].queue;
        // persistent groups (with a queue): a group takes the next geometry
        // from the queue when it finishes one, so uneven geometries balance at
        // the granularity of one geometry (not of a CTA's G geometries);
        // without a queue (and always for tcgen05), one geometry per group
        const bool persistent = ENG != ENG_TC && queue != nullptr;
        __shared__ int next_th[8];
        for (int round = 0;; ++round) {
            int th;
            if (persistent) {
                if (grp.gt == 0) next_th[grp.id] = atomicAdd(queue, 1);
                grp.sync();
                th = next_th[grp.id];
                grp.sync();
            } else {
                if (round > 0) break;
                th = blockIdx.x * G + grp.id;
            }
            if (th >= ntot) break;
            // the part that holds queue index th (parts are few: a linear scan)
            int p = 0;
            while (p + 1 < P.n && th >= P.start[p + 1]) ++p;
            group_body<T, RT, ENG, WG>(P.m[p], P.a[p], grp, th - P.start[p], gsm, tmem_base);
            grp.sync();
        }
    }
    if constexpr (ENG == ENG_TC) {
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (warp == 0) tc::tmem_dealloc(tmem_base, ncols);
    }
}

template <typename T, int RT, int ENG, int WG>
__global__ void __launch_bounds__(is_mma(ENG) ? 512 : 256) inner_group_kernel(const __grid_constant__ InnerParts P,
                                                                               int W, int G) {
    inner_group_entry<T, RT, ENG, WG>(P, W, G);
}

// the global-matrix engine: one 512-thread CTA per SM, so up to 128 registers
// per thread for the positions, momenta and products of its rows and slots
template <typename T, int RT>
__global__ void __launch_bounds__(512, 1) inner_gl_kernel(const __grid_constant__ InnerParts P) {
    inner_group_entry<T, RT, ENG_GL, 16>(P, 16, 1);
}

// CTAs of a persistent launch: one wave (resident CTAs), no more than the
// geometries need, but one CTA per SM as long as there are at least as many
// geometries as SMs (a batch of 500 geometries in CTAs of four groups then
// spreads over all 152 SMs instead of filling 125); the queue counter is
// reset on the launch's stream.  Without a queue, one CTA per G geometries.
static unsigned persistent_blocks(const InnerParts &P, int G, int resident, cudaStream_t s) {
    const int ntot = P.start[P.n];
    int need = (ntot + G - 1) / G;
    int *queue = P.a[0].queue;
    if (!queue) return (unsigned)need;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    need = std::max(need, std::min(ntot, nsm));
    if (cudaMemsetAsync(queue, 0, sizeof(int), s) != cudaSuccess) return 0;
    return (unsigned)std::max(1, std::min(need, resident));
}

template <typename T, int RT>
static cudaError_t launch_cc_t(const InnerParts &P, cudaStream_t s, int W) {
    using L_ = Layout<T, RT, ENG_CC>;
    int dev = 0, maxsm = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int ntot = P.start[P.n];
    if (W <= 0) {
        // warps per geometry from the batch size: enough geometries in flight
        // to fill every SM with 8 warps, otherwise more slots per geometry
        const long long slots = 8LL * nsm;
        W = 1;
        while (W < 8 && (long long)ntot * W * 2 <= slots) W *= 2;
    }
    size_t per = L_::bytes(W);
    int G = (int)std::min<size_t>((size_t)(8 / W), (size_t)maxsm / per);
    while (G < 1 && W > 1) {
        W /= 2;
        per = L_::bytes(W);
        G = (int)std::min<size_t>((size_t)(8 / W), (size_t)maxsm / per);
    }
    if (G < 1) return cudaErrorInvalidValue;
    size_t sm = per * G;
    cudaError_t e = cudaFuncSetAttribute(inner_group_kernel<T, RT, ENG_CC, 0>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, inner_group_kernel<T, RT, ENG_CC, 0>, 32 * W * G, sm);
    if (e != cudaSuccess) return e;
    const unsigned blocks = persistent_blocks(P, G, nsm * std::max(occ, 1), s);
    if (!blocks) return cudaGetLastError();
    inner_group_kernel<T, RT, ENG_CC, 0><<<blocks, 32 * W * G, sm, s>>>(P, W, G);
    return cudaGetLastError();
}

// WG warps per geometry: as many geometries per CTA as shared memory and the
// register file allow (gmax), but no more than needed to give every SM a CTA
template <int RT, int ENG, int WG>
static cudaError_t launch_wg_t(const InnerParts &P, cudaStream_t s, int gmax) {
    using L_ = Layout<float, RT, ENG>;
    int dev = 0, maxsm = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int ntot = P.start[P.n];
    const size_t per = L_::bytes(WG);
    int G = (int)std::min<size_t>((size_t)gmax, (size_t)maxsm / per);
    G = std::min(G, std::max(1, (ntot + nsm - 1) / nsm));
    if (G < 1) return cudaErrorInvalidValue;
    const size_t sm = per * G;
    cudaError_t e = cudaFuncSetAttribute(inner_group_kernel<float, RT, ENG, WG>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    unsigned blocks = (unsigned)((ntot + G - 1) / G);
    if (ENG != ENG_TC) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, inner_group_kernel<float, RT, ENG, WG>, 32 * WG * G, sm);
        if (e != cudaSuccess) return e;
        blocks = persistent_blocks(P, G, nsm * std::max(occ, 1), s);
        if (!blocks) return cudaGetLastError();
    }
    inner_group_kernel<float, RT, ENG, WG><<<blocks, 32 * WG * G, sm, s>>>(P, WG, G);
    return cudaGetLastError();
}

// Global-matrix engine: one geometry per CTA of 16 warps, persistent over the
// batch (a CTA takes the next geometry from the queue when it finishes one).
template <typename T, int RT>
static cudaError_t launch_gl_t(const InnerParts &P, cudaStream_t s) {
    using L_ = Layout<T, RT, ENG_GL>;
    constexpr int WG = 16;
    for (int p = 0; p < P.n; ++p) {
        const InnerArgs &a = P.a[p];
        if (a.D > L_::DP || !a.mgl || !a.glxc) return cudaErrorInvalidValue;
        if (!std::is_same<T, double>::value && !a.A32) return cudaErrorInvalidValue;
    }
    if (!P.a[0].queue) return cudaErrorInvalidValue;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t sm = L_::bytes(WG);
    cudaError_t e = cudaFuncSetAttribute(inner_gl_kernel<T, RT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, inner_gl_kernel<T, RT>, 32 * WG, sm);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const unsigned blocks = persistent_blocks(P, 1, nsm * occ, s);
    if (!blocks) return cudaGetLastError();
    inner_gl_kernel<T, RT><<<blocks, 32 * WG, sm, s>>>(P);
    return cudaGetLastError();
}

}  // namespace smc
