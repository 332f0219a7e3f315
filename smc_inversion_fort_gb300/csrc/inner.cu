// Inner tempered SMC over slip on the GPU: one CTA per geometry particle,
// persistent across all tempering stages (slip_smc_exec,
// smc_slip.f90:1445-1663).
//
// HMC children of one parent form a Metropolis chain (slip_hmc_sampling,
// smc_slip.f90:591-730): child k starts from the state left by child k-1.
// The CTA runs C chain slots in lock step; a slot works through one parent's
// children, then takes the next parent from a queue ordered by descending
// child count (longest chains first).  Every leapfrog step of all slots is one
// small GEMM  grad = M x  (M = gamma*A + L^T L / alpha^2, x the D x C tile
// of slot positions) held in shared memory; each thread owns an RT x CT block
// of rows x slots and applies the position/momentum update, the reflection at
// [0, max_slip] and the blow-up test element-wise.  Random draws are addressed
// by (stage, purpose, child index, dimension), so the result does not depend
// on which slot runs which chain.
//
// Precision modes.  FP64 (T = double): the reference's algebra in FP64,
// grad = gamma (A x - b) + L^T (L x)/alpha^2 folded as M x - gamma b,
// likelihood by the Gram form (smc_slip.f90:56-104), prior by the sparse L
// (smc_slip.f90:106-137).  MIXED (T = float): leapfrog in FP32 about the
// stage mean sbar, grad = c + M (x - sbar) with c = gamma (A sbar - b) +
// L^T L sbar/alpha^2 in FP64; trajectory end points are scored in FP64 as
// L(sbar) + g.delta + delta.A.delta/2 and P(sbar) + h.delta + |L delta|^2/(2 alpha^2),
// which keeps the Gram form's cancellation out of FP32.
#include <type_traits>

#include "common.cuh"
#include "ddreal.cuh"
#include "inner.h"
#include "q128.cuh"

namespace smc {

constexpr int NT = 256;
constexpr int TYN = 16, TXN = 16;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ double block_sum(double v, double *scr) {
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) scr[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) t += scr[i];
    return t;
}
__device__ double block_min(double v, double *scr) {
    v = warp_min(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) scr[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = scr[0];
#pragma unroll
    for (int i = 1; i < NT / 32; ++i) t = fmin(t, scr[i]);
    return t;
}
__device__ dd block_sum_dd(dd v, dd *scr) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dd n = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = dd_add(v, n);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) scr[threadIdx.x >> 5] = v;
    __syncthreads();
    dd t = scr[0];
#pragma unroll
    for (int i = 1; i < NT / 32; ++i) t = dd_add(t, scr[i]);
    return t;
}
// exclusive scan of one int per thread over the block; returns the prefix,
// total via reference
__device__ int block_exscan(int v, int *scr, int &total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += n;
    }
    __syncthreads();
    if (lane == 31) scr[wid] = x;
    __syncthreads();
    int base = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) {
        if (i < wid) base += scr[i];
        tot += scr[i];
    }
    total = tot;
    return base + x - v;
}

// w / (s.hi + s.lo) rounded to double: the binary128 division of
// slip_normalize_weights (smc_slip.f90:465-483) to within an ulp
__device__ __forceinline__ double dd_div_into(double w, dd s) {
    double q = w / s.hi;
    double r = fma(-q, s.hi, w) - q * s.lo;
    return q + r / s.hi;
}

// Reflection into [0, max_slip] with momentum flips (smc_slip.f90:787-799).
template <typename T>
__device__ __forceinline__ void reflect(T &x, T &p, T mx, int &flag) {
    int it = 0;
    while (x < T(0) || x > mx) {
        if (x > mx) { x = T(2) * mx - x; p = -p; }
        if (x < T(0)) { x = -x; p = -p; }
        if (++it > 1000000) { flag |= SMCGPU_ST_REFLECT_CAP; break; }
    }
}

// Residual-systematic counts of w[0..n) with multiplier count_n (scan form,
// resample.cu); writes cnt[i] and returns the total.
__device__ long long scan_counts(const double *w, int n, int count_n, double u_hi, double u_lo, int *cnt,
                                 dd *ddscr, long long *llscr, int *s_tie) {
    if (threadIdx.x == 0) *s_tie = 0;
    __syncthreads();
    dd carry = {0.0, 0.0};
    long long prevC = 0;
    const dd u0 = {u_hi, u_lo};
    const double dn = (double)count_n;
    for (int base = 0; base < n; base += NT) {
        int i = base + threadIdx.x;
        dd v = {i < n ? w[i] : 0.0, 0.0};
        dd tot;
        dd incl = block_scan_dd(v, ddscr, tot);
        incl = dd_add(carry, incl);
        carry = dd_add(carry, tot);
        dd x = dd_add(dd_mul_d(incl, dn), dd_neg(u0));
        double frac;
        long long C = dd_floor(x, frac) + 1;
        if (i < n && (frac < 1e-20 || frac > 1.0 - 1e-20)) *s_tie = 1;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        long long Cp = __shfl_up_sync(0xffffffffu, C, 1);
        if (lane == 31) llscr[wid] = C;
        __syncthreads();
        if (lane == 0) Cp = wid == 0 ? prevC : llscr[wid - 1];
        if (i < n) cnt[i] = (int)(C - Cp);
        prevC = llscr[NT / 32 - 1];
        __syncthreads();
    }
    if (*s_tie) {
        if (threadIdx.x == 0) {
            q128 dnq = q128_from_int(count_n);
            q128 u = q128_div(q128_add(q128_from_double(u_hi), q128_from_double(u_lo)), dnq);
            for (int i = 0; i < n; ++i) {
                q128 wi = q128_from_double(w[i]);
                long long aq = q128_floor(q128_mul(q128_sub(wi, u), dnq)) + 1;
                cnt[i] = (int)aq;
                u = q128_sub(q128_add(u, q128_div(q128_from_int(aq), dnq)), wi);
            }
        }
        __syncthreads();
        long long t = 0;
        for (int i = 0; i < n; ++i) t += cnt[i];
        return t;
    }
    return prevC;
}

// ---------------------------------------------------------------------------
// Truncated-normal Gibbs initialisation (slip_gen_init_particles,
// smc_slip.f90:184-264): one warp per geometry runs the reference's single
// chained sweep (particle k is one sweep after particle k-1, starting at 0).
// FP64 uses the reference's Newton inverse CDF; MIXED inverts in FP32
// through normcdff/normcdfinvf on the tail-appropriate side.
// ---------------------------------------------------------------------------
template <bool MIXED>
__global__ void gibbs_kernel(MeshDev m, InnerArgs a) {
    extern __shared__ double gsh[];
    const int wpb = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int th = blockIdx.x * wpb + wid;
    if (th >= a.n_theta) return;
    const int D = a.D, N = a.N;
    double *cur = gsh + (size_t)wid * 2 * D, *vn = cur + D;
    const double alpha2 = a.aux[th].alpha2;
    const double *ll = a.llval + (size_t)th * m.ll_nnz;
    const uint64_t stream = a.streams[th];
    double *parts = a.parts + (size_t)th * N * D;
    int stat = 0;
    for (int i = lane; i < D; i += 32) cur[i] = 0.0;
    __syncwarp();
    const double pi = 3.141592653589793;
    for (int k = 0; k < N; ++k) {
        for (int d = lane; d < D; d += 32)
            vn[d] = MIXED ? (double)rng_normal_f(a.seed, stream, RNG_GIBBS, 0, k, d)
                          : rng_normal(a.seed, stream, RNG_GIBBS, 0, k, d);
        __syncwarp();
        for (int i = 0; i < D; ++i) {
            int e0 = m.ll_ptr[i], e1 = m.ll_ptr[i + 1];
            // diagonal entry and the conditional mean
            int e = e0 + lane;
            int j = e < e1 ? m.ll_col[e] : -1;
            double v = e < e1 ? ll[e] : 0.0;
            double s2, mu;
            if (!MIXED) {
                double lii = (j == i) ? v : 0.0, term = 0.0;
                lii = warp_sum(lii);
                s2 = 1.0 / (lii / alpha2);
                if (j >= 0 && j != i) term = v / alpha2 * cur[j] * s2;
                mu = -warp_sum(term);
            } else {
                float lii = (j == i) ? (float)v : 0.0f, term = 0.0f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) lii += __shfl_xor_sync(0xffffffffu, lii, o);
                if (j >= 0 && j != i) term = (float)v * (float)cur[j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
                float s2f = (float)alpha2 / lii;
                s2 = (double)s2f;
                mu = (double)(-term / lii);
            }
            if (lane == 0) {
                double v1 = vn[i];
                double y;
                if (!MIXED) {
                    double sq = sqrt(2.0 * s2), pdfn = sqrt(2.0 * pi * s2);
                    double x = mu + v1 * sqrt(s2);
                    double fx = (1.0 + erf((x - mu) / sq)) / 2.0;
                    double f1 = (1.0 + erf((a.max_slip - mu) / sq)) / 2.0;
                    double f0 = (1.0 + erf((0.0 - mu) / sq)) / 2.0;
                    double target = (f1 - f0) * fx + f0;
                    y = mu;
                    double err = 1.0, yp = y + err;
                    int cnt = 0;
                    while (err > 1e-8 && cnt < 100) {
                        double cdf = (1.0 + erf((y - mu) / sq)) / 2.0;
                        double pdf = exp(-((y - mu) * (y - mu)) / (2.0 * s2)) / pdfn;
                        y = y - (cdf - target) / pdf;
                        err = fabs(y - yp);
                        yp = y;
                        ++cnt;
                    }
                    if (cnt >= 100) stat |= SMCGPU_ST_NEWTON_CAP;
                } else {
                    float sg = sqrtf((float)s2), muf = (float)mu;
                    float al = (0.0f - muf) / sg, be = ((float)a.max_slip - muf) / sg;
                    float u = normcdff((float)v1);
                    float z;
                    if (al >= 0.0f) {
                        float qa = normcdff(-al), qb = normcdff(-be);
                        float q = qa - u * (qa - qb);
                        z = q > 0.0f ? -normcdfinvf(q) : al;
                    } else {
                        float pa = normcdff(al), pb = normcdff(be);
                        float p = pa + u * (pb - pa);
                        z = p > 0.0f ? normcdfinvf(p) : be;
                    }
                    float yf = muf + sg * z;
                    yf = fminf(fmaxf(yf, 0.0f), (float)a.max_slip);
                    y = (double)yf;
                }
                cur[i] = y;
            }
            __syncwarp();
        }
        for (int d = lane; d < D; d += 32) parts[(size_t)k * D + d] = cur[d];
        __syncwarp();
    }
    if (lane == 0 && stat) atomicOr(a.status + th, stat);
}

// ---------------------------------------------------------------------------
// Main kernel
// ---------------------------------------------------------------------------
template <typename T, int RT, int CT>
struct Tile {
    static constexpr int DP = TYN * RT;   // padded dimension
    static constexpr int C = TXN * CT;    // chain slots
};

template <typename T, int RT, int CT>
__device__ __forceinline__ void tile_gemm(const T *__restrict__ Mcol, const T *__restrict__ X, int ty, int tx,
                                          T acc[RT][CT]) {
    constexpr int DP = Tile<T, RT, CT>::DP, C = Tile<T, RT, CT>::C;
#pragma unroll
    for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int q = 0; q < CT; ++q) acc[i][q] = T(0);
    const T *mp = Mcol + ty * RT;
    const T *xp = X + tx * CT;
#pragma unroll 4
    for (int k = 0; k < DP; ++k) {
        T mv[RT], xv[CT];
#pragma unroll
        for (int i = 0; i < RT; ++i) mv[i] = mp[(size_t)k * DP + i];
#pragma unroll
        for (int q = 0; q < CT; ++q) xv[q] = xp[(size_t)k * C + q];
#pragma unroll
        for (int i = 0; i < RT; ++i)
#pragma unroll
            for (int q = 0; q < CT; ++q) acc[i][q] = fma(mv[i], xv[q], acc[i][q]);
    }
}

struct SlotState {
    int *par, *j, *jend, *fresh, *blown, *acc;
    double *L, *P, *post, *ham, *dt, *Lx, *Px, *K, *S;
};

template <typename T, int RT, int CT>
__global__ void __launch_bounds__(NT, 1) inner_kernel(MeshDev m, InnerArgs a) {
    using TL = Tile<T, RT, CT>;
    constexpr int DP = TL::DP, C = TL::C;
    constexpr bool MIXED = std::is_same<T, float>::value;
    const int th = blockIdx.x;
    if (th >= a.n_theta) return;
    const int N = a.N, D = a.D, NP2 = a.NP2;
    const int tid = threadIdx.x, ty = tid / TXN, tx = tid % TXN;

    extern __shared__ __align__(16) unsigned char smem[];
    T *Msm = (T *)smem;                          // DP*DP, column-major
    T *Asm = Msm + DP * DP;                      // DP*DP
    T *Xb0 = Asm + DP * DP;                      // DP*C
    T *Xb1 = Xb0 + DP * C;
    // per-row constants of the stage in the leapfrog's own precision, so the
    // step loop never touches the FP64 pipe in MIXED mode
    T *tcov = Xb1 + DP * C, *tmean = tcov + DP, *tcv = tmean + DP, *tisc = tcv + DP;
    double *vb = (double *)(tisc + DP);          // b
    double *vcov = vb + DP, *vmean = vcov + DP, *vg = vmean + DP, *vh = vg + DP, *vc = vh + DP;
    double *red = vc + DP;                       // TYN*C
    double *scr = red + TYN * C;                 // 64 doubles (also 32 dd)
    double *sd = scr + 64;                       // slot doubles: 9*C
    int *si = (int *)(sd + 9 * C);               // slot ints: 6*C
    long long *llscr = (long long *)(si + 6 * C + (6 * C) % 2);
    SlotState s;
    s.L = sd; s.P = sd + C; s.post = sd + 2 * C; s.ham = sd + 3 * C; s.dt = sd + 4 * C;
    s.Lx = sd + 5 * C; s.Px = sd + 6 * C; s.K = sd + 7 * C; s.S = sd + 8 * C;
    s.par = si; s.j = si + C; s.jend = si + 2 * C; s.fresh = si + 3 * C; s.blown = si + 4 * C; s.acc = si + 5 * C;
    __shared__ int s_status, s_tie, s_next, s_any, s_qlen;
    __shared__ double s_Lbar, s_Pbar;

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
    const T mx = (T)a.max_slip;

    if (tid == 0) s_status = 0;
    // constants into shared memory (zero padded)
    for (int e = tid; e < DP * DP; e += NT) {
        int i = e % DP, k = e / DP;
        Asm[e] = (i < D && k < D) ? (T)Ath[(size_t)k * D + i] : T(0);
    }
    for (int i = tid; i < DP; i += NT) vb[i] = i < D ? bth[i] : 0.0;
    for (int k = tid; k < N; k += NT) dtau[k] = exp(-5.0);
    __syncthreads();

    // likelihood and prior of the initial particles, FP64 Gram form
    {
        const int wid = tid >> 5, lane = tid & 31;
        for (int k = wid; k < N; k += NT / 32) {
            const double *x = parts + (size_t)k * D;
            double qa = 0.0, bx = 0.0;
            for (int i = lane; i < D; i += 32) {
                double t = 0.0;
                for (int j2 = 0; j2 < D; ++j2) t += Ath[(size_t)j2 * D + i] * x[j2];
                qa += x[i] * t;
                bx += vb[i] * x[i];
            }
            qa = warp_sum(qa);
            bx = warp_sum(bx);
            double pr = 0.0;
            for (int r = lane; r < m.nrow; r += 32) {
                double t = 0.0;
                for (int q = 0; q < 9; ++q) {
                    int c = m.l_col[r * 9 + q];
                    if (c >= 0) t += lv[(size_t)r * 9 + q] * x[c];
                }
                pr += t * t / (2.0 * alpha2);
            }
            pr = warp_sum(pr);
            if (lane == 0) {
                Lc[k] = (qa - 2.0 * bx + dsd) / 2.0 + lconst;
                Pc[k] = pr;
            }
        }
    }
    __syncthreads();

    double gamma = 0.0, neglog = 0.0, log_up = 0.0, log_lo = -1e1;
    int iter = 1;
    while (1.0 - gamma > 10e-8) {
        // ---- slip_find_next_gamma (smc_slip.f90:314-387)
        double lmin = 1e300;
        for (int k = tid; k < N; k += NT) lmin = fmin(lmin, Lc[k]);
        lmin = block_min(lmin, scr);
        const double gprev = gamma;
        double lower = gprev, upper = 1.0, err = 1.0, g = 1.0;
        int bcnt = 0;
        while (err > 1e-10) {
            g = (lower + upper) / 2.0;
            double dg = g - gprev, ps = 0.0;
            for (int k = tid; k < N; k += NT) {
                double wk = exp(-dg * (Lc[k] - lmin));
                w[k] = wk;
                ps += wk;
            }
            double mean = block_sum(ps, scr) / N;
            double pv = 0.0;
            for (int k = tid; k < N; k += NT) {
                double dv = w[k] - mean;
                pv += dv * dv;
            }
            double sdv = sqrt(block_sum(pv, scr) / N);
            double cv = sdv / mean;
            if (cv > a.cv) upper = g; else lower = g;
            err = fabs(cv - a.cv);
            if (fabs(g - 1.0) < 1e-10) break;
            if (++bcnt > 2000) {
                if (tid == 0) atomicOr(&s_status, SMCGPU_ST_BISECT_CAP);
                break;
            }
        }
        double dg = g - gprev, ps = 0.0;
        for (int k = tid; k < N; k += NT) ps += exp(-dg * (Lc[k] - lmin));
        double ev = block_sum(ps, scr) / N;
        double inc = -log(ev) + dg * lmin;
        gamma = g;
        neglog += inc;
        if (tid == 0 && a.trace_gamma) {
            a.trace_gamma[(size_t)th * (a.max_stages + 2) + iter - 1] = gamma;
            a.trace_inc[(size_t)th * (a.max_stages + 2) + iter - 1] = inc;
        }
        if (iter > a.max_stages) {
            neglog = 1e10;
            if (tid == 0) atomicOr(&s_status, SMCGPU_ST_STAGE_CAP);
            break;
        }
        // ---- normalise, mean, diagonal covariance (smc_slip.f90:465-570)
        {
            dd ps2 = {0.0, 0.0};
            for (int k = tid; k < N; k += NT) ps2 = dd_add_d(ps2, w[k]);
            dd sw = block_sum_dd(ps2, (dd *)scr);
            __syncthreads();
            for (int k = tid; k < N; k += NT) w[k] = dd_div_into(w[k], sw);
            __syncthreads();
        }
        for (int d = tid; d < DP; d += NT) {
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
                double md = 0.0;
                for (int k = 0; k < N; ++k) md += w[k] * parts[(size_t)k * D + d];
                double cd = 0.0;
                for (int k = 0; k < N; ++k) {
                    double di = parts[(size_t)k * D + d] - md;
                    cd += w[k] * di * di;
                }
                vmean[d] = md;
                vcov[d] = fabs(cd) < 1e-3 ? 1e-3 : cd;
            }
        }
        // ---- resampling counts (smc_slip.f90:572-589) and child offsets
        {
            double uh, ul;
            rng_quad_uniform(a.seed, stream, RNG_RESAMPLE, iter, uh, ul);
            __syncthreads();
            scan_counts(w, N, N, uh, ul, cnt, (dd *)scr, llscr, &s_tie);
            __syncthreads();
            int carry = 0;
            for (int base = 0; base < N; base += NT) {
                int k = base + tid;
                int v = k < N ? cnt[k] : 0, tot;
                int ex = block_exscan(v, (int *)scr, tot);
                if (k < N) ids[k] = carry + ex;
                carry += tot;
            }
            __syncthreads();
        }
        // ---- stage matrices: M = gamma A + L^T L/alpha^2 (FP64 mode) and,
        // in MIXED, the centring terms at the weighted mean
        for (int e = tid; e < DP * DP; e += NT) {
            int i = e % DP, k = e / DP;
            Msm[e] = (i < D && k < D) ? (T)(gamma * Ath[(size_t)k * D + i]) : T(0);
        }
        __syncthreads();
        for (int i = tid; i < D; i += NT) {
            for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) {
                int k = m.ll_col[e];
                Msm[(size_t)k * DP + i] = (T)((double)Msm[(size_t)k * DP + i] + llv[e] / alpha2);
            }
        }
        if (MIXED) {
            __syncthreads();
            // g = A sbar - b, h = L^T L sbar / alpha^2, c = gamma g + h
            for (int i = tid; i < DP; i += NT) {
                double gi = 0.0, hi = 0.0;
                if (i < D) {
                    for (int k = 0; k < D; ++k) gi += Ath[(size_t)k * D + i] * vmean[k];
                    gi -= vb[i];
                    for (int e = m.ll_ptr[i]; e < m.ll_ptr[i + 1]; ++e) hi += llv[e] * vmean[m.ll_col[e]];
                    hi /= alpha2;
                }
                vg[i] = gi;
                vh[i] = hi;
                vc[i] = gamma * gi + hi;
            }
            // L(sbar) (Gram form) and P(sbar)
            double qa = 0.0, bx = 0.0, pr = 0.0;
            for (int i = tid; i < D; i += NT) {
                double t = 0.0;
                for (int k = 0; k < D; ++k) t += Ath[(size_t)k * D + i] * vmean[k];
                qa += vmean[i] * t;
                bx += vb[i] * vmean[i];
            }
            for (int r = tid; r < m.nrow; r += NT) {
                double t = 0.0;
                for (int q = 0; q < 9; ++q) {
                    int c = m.l_col[r * 9 + q];
                    if (c >= 0) t += lv[(size_t)r * 9 + q] * vmean[c];
                }
                pr += t * t / (2.0 * alpha2);
            }
            qa = block_sum(qa, scr);
            bx = block_sum(bx, scr);
            pr = block_sum(pr, scr);
            if (tid == 0) {
                s_Lbar = (qa - 2.0 * bx + dsd) / 2.0 + lconst;
                s_Pbar = pr;
            }
        }
        for (int i = tid; i < DP; i += NT) {
            tcov[i] = (T)vcov[i];
            tmean[i] = (T)vmean[i];
            tcv[i] = MIXED ? (T)vc[i] : (T)(gamma * vb[i]);
            tisc[i] = (T)(1.0 / sqrt(vcov[i]));
        }
        __syncthreads();

        // ---- one HMC pass: tuning (every tf-th parent) or sampling
        for (int pass = 0; pass < 2; ++pass) {
            const bool tuning = pass == 0;
            const uint32_t P_MOM = tuning ? RNG_TUNE_MOM : RNG_SMP_MOM;
            const uint32_t P_MH = tuning ? RNG_TUNE_MH : RNG_SMP_MH;
            // parent queue, longest chains first
            int nq_local = 0;
            for (int k = tid; k < NP2; k += NT) {
                bool ok = k < N && cnt[k] > 0 && (!tuning || k % a.tf == 0);
                keys[k] = ok ? (int)(((unsigned)(N - cnt[k]) << 16) | (unsigned)k) : 0x7fffffff;
                nq_local += ok;
            }
            int nq = (int)block_sum((double)nq_local, scr);
            __syncthreads();
            for (int size = 2; size <= NP2; size <<= 1)
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int i = tid; i < NP2; i += NT) {
                        int jx = i ^ stride;
                        if (jx > i) {
                            int ka = keys[i], kb = keys[jx];
                            bool up = (i & size) == 0;
                            if ((ka > kb) == up) { keys[i] = kb; keys[jx] = ka; }
                        }
                    }
                    __syncthreads();
                }
            // no tuned child: step sizes stay as they are (smc_slip.f90:993-995)
            if (tuning && nq == 0) continue;
            if (tuning) {
                // step sizes of the tuned children (smc_slip.f90:979-992)
                for (int q = tid; q < nq; q += NT) {
                    int k = keys[q] & 0xffff;
                    for (int jj = ids[k]; jj < ids[k] + cnt[k]; ++jj) {
                        double ld = rng_uniform(a.seed, stream, RNG_TUNE_DTAU, iter, jj, 0);
                        ld = log_lo + ld * (log_up - log_lo);
                        dtau[jj] = exp(ld);
                    }
                }
            }
            if (tid == 0) { s_next = 0; s_qlen = nq; }
            for (int c = tid; c < C; c += NT) { s.j[c] = 0; s.jend[c] = 0; s.par[c] = -1; }
            __syncthreads();

            T xc[RT][CT], x[RT][CT], p[RT][CT], acc[RT][CT];
#pragma unroll
            for (int i = 0; i < RT; ++i)
#pragma unroll
                for (int q = 0; q < CT; ++q) xc[i][q] = T(0);
            while (true) {
                if (tid == 0) {
                    int any = 0;
                    for (int c = 0; c < C; ++c) {
                        s.fresh[c] = 0;
                        if (s.j[c] >= s.jend[c] && s_next < s_qlen) {
                            int k = keys[s_next++] & 0xffff;
                            s.par[c] = k;
                            s.j[c] = ids[k];
                            s.jend[c] = ids[k] + cnt[k];
                            s.fresh[c] = 1;
                        }
                        any |= s.j[c] < s.jend[c];
                    }
                    s_any = any;
                }
                __syncthreads();
                if (!s_any) break;
                // slot set-up: parent state for fresh slots, step size, momenta
                if (tid < C) {
                    int c = tid;
                    if (s.fresh[c]) {
                        int k = s.par[c];
                        s.L[c] = Lc[k];
                        s.P[c] = Pc[k];
                        s.post[c] = gamma * Lc[k] + Pc[k];
                    }
                    bool act = s.j[c] < s.jend[c];
                    s.dt[c] = act ? dtau[s.j[c]] : 0.0;
                    s.blown[c] = 0;
                }
                __syncthreads();
                double kin[CT];
#pragma unroll
                for (int q = 0; q < CT; ++q) {
                    int c = tx * CT + q;
                    bool act = s.j[c] < s.jend[c];
                    kin[q] = 0.0;
#pragma unroll
                    for (int i = 0; i < RT; ++i) {
                        int r = ty * RT + i;
                        if (s.fresh[c]) xc[i][q] = (act && r < D) ? (T)parts[(size_t)s.par[c] * D + r] : T(0);
                        T pv = T(0);
                        if (act && r < D) {
                            if (MIXED) {
                                pv = rng_normal_f(a.seed, stream, P_MOM, iter, s.j[c], r) * tisc[r];
                                kin[q] += (double)(pv * tcov[r] * pv * T(0.5));
                            } else {
                                pv = (T)(rng_normal(a.seed, stream, P_MOM, iter, s.j[c], r) / sqrt(vcov[r]));
                                kin[q] += (double)pv * vcov[r] * (double)pv / 2.0;
                            }
                        }
                        p[i][q] = pv;
                        x[i][q] = xc[i][q];
                        T xv = MIXED ? x[i][q] - tmean[r] : x[i][q];
                        Xb0[(size_t)r * C + c] = (r < D) ? xv : T(0);
                    }
                    red[ty * C + c] = kin[q];
                }
                __syncthreads();
                if (tid < C) {
                    double t = 0.0;
                    for (int y2 = 0; y2 < TYN; ++y2) t += red[y2 * C + tid];
                    s.ham[tid] = s.post[tid] + t;
                }
                // leapfrog (smc_slip.f90:755-904): P/2 (X P)^ntau X/2
                int flag = 0;
                T dts[CT];
#pragma unroll
                for (int q = 0; q < CT; ++q) dts[q] = (T)s.dt[tx * CT + q];
                for (int it = 0; it <= a.ntau; ++it) {
                    T *Xr = (it & 1) ? Xb1 : Xb0;
                    T *Xw = (it & 1) ? Xb0 : Xb1;
                    tile_gemm<T, RT, CT>(Msm, Xr, ty, tx, acc);
                    const T hstep = (it == 0) ? T(0.5) : T(1);
#pragma unroll
                    for (int q = 0; q < CT; ++q) {
                        int c = tx * CT + q;
                        bool live = s.j[c] < s.jend[c] && !s.blown[c];
#pragma unroll
                        for (int i = 0; i < RT; ++i) {
                            int r = ty * RT + i;
                            if (!live || r >= D) continue;
                            T gr = MIXED ? tcv[r] + acc[i][q] : acc[i][q] - tcv[r];
                            p[i][q] = p[i][q] - gr * hstep * dts[q];
                        }
                    }
                    // position step (full, or the final half step)
                    const T xstep = (it == a.ntau) ? T(0.5) : T(1);
#pragma unroll
                    for (int q = 0; q < CT; ++q) {
                        int c = tx * CT + q;
                        bool live = s.j[c] < s.jend[c] && !s.blown[c];
#pragma unroll
                        for (int i = 0; i < RT; ++i) {
                            int r = ty * RT + i;
                            if (live && r < D) {
                                x[i][q] = x[i][q] + tcov[r] * p[i][q] * xstep * dts[q];
                                if (fabs(x[i][q]) > T(1e3)) atomicOr(&s.blown[c], 1);
                                else reflect<T>(x[i][q], p[i][q], mx, flag);
                            }
                            T xv = MIXED ? x[i][q] - tmean[r] : x[i][q];
                            Xw[(size_t)r * C + c] = (r < D) ? xv : T(0);
                        }
                    }
                    __syncthreads();
                }
                if (flag) atomicOr(&s_status, flag);
                // trajectory end point: likelihood, prior, kinetic energy (and score)
                {
                    T *Xf = ((a.ntau + 1) & 1) ? Xb1 : Xb0;
                    tile_gemm<T, RT, CT>(Asm, Xf, ty, tx, acc);
                    double pl[CT], pk[CT], psc[CT];
#pragma unroll
                    for (int q = 0; q < CT; ++q) {
                        int c = tx * CT + q;
                        pl[q] = pk[q] = psc[q] = 0.0;
#pragma unroll
                        for (int i = 0; i < RT; ++i) {
                            int r = ty * RT + i;
                            if (r >= D) continue;
                            if (MIXED) {
                                double del = (double)x[i][q] - vmean[r];
                                pl[q] += vg[r] * del + 0.5 * (double)Xf[(size_t)r * C + c] * (double)acc[i][q];
                            } else {
                                double xv = (double)x[i][q];
                                pl[q] += xv * (double)acc[i][q] - 2.0 * vb[r] * xv;
                            }
                            pk[q] += (double)p[i][q] * vcov[r] * (double)p[i][q] / 2.0;
                            double dx = (double)x[i][q] - (double)xc[i][q];
                            psc[q] += dx * dx / vcov[r];
                        }
                    }
                    // sums over row groups, one quantity at a time
                    for (int qq = 0; qq < 3; ++qq) {
#pragma unroll
                        for (int q = 0; q < CT; ++q)
                            red[ty * C + tx * CT + q] = qq == 0 ? pl[q] : (qq == 1 ? pk[q] : psc[q]);
                        __syncthreads();
                        if (tid < C) {
                            double t = 0.0;
                            for (int y2 = 0; y2 < TYN; ++y2) t += red[y2 * C + tid];
                            if (qq == 0) s.Lx[tid] = t;
                            else if (qq == 1) s.K[tid] = t;
                            else s.S[tid] = t;
                        }
                        __syncthreads();
                    }
                    // prior through the sparse L rows (FP64 mode: of x, MIXED: of delta)
                    double pp[CT];
#pragma unroll
                    for (int q = 0; q < CT; ++q) {
                        int c = tx * CT + q;
                        pp[q] = 0.0;
                        for (int r = ty; r < m.nrow; r += TYN) {
                            double t = 0.0;
                            for (int k9 = 0; k9 < 9; ++k9) {
                                int cl = m.l_col[r * 9 + k9];
                                if (cl >= 0) t += lv[(size_t)r * 9 + k9] * (double)Xf[(size_t)cl * C + c];
                            }
                            pp[q] += t * t / (2.0 * alpha2);
                        }
                        red[ty * C + c] = pp[q];
                    }
                    __syncthreads();
                    if (tid < C) {
                        double t = 0.0;
                        for (int y2 = 0; y2 < TYN; ++y2) t += red[y2 * C + tid];
                        s.Px[tid] = t;
                    }
                    if (MIXED) {
                        // linear terms of the prior expansion
                        __syncthreads();
#pragma unroll
                        for (int q = 0; q < CT; ++q) {
                            int c = tx * CT + q;
                            double t = 0.0;
#pragma unroll
                            for (int i = 0; i < RT; ++i) {
                                int r = ty * RT + i;
                                if (r < D) t += vh[r] * ((double)x[i][q] - vmean[r]);
                            }
                            red[ty * C + c] = t;
                        }
                        __syncthreads();
                        if (tid < C) {
                            double t = 0.0;
                            for (int y2 = 0; y2 < TYN; ++y2) t += red[y2 * C + tid];
                            s.Px[tid] += t + s_Pbar;
                            s.Lx[tid] += s_Lbar;
                        }
                    }
                    __syncthreads();
                }
                // Metropolis test and bookkeeping (smc_slip.f90:695-716, 1057-1094)
                if (tid < C) {
                    int c = tid;
                    s.acc[c] = 0;
                    if (s.j[c] < s.jend[c]) {
                        int jj = s.j[c];
                        double Lx, Px, post, ham;
                        if (s.blown[c]) {
                            ham = 1e20;
                            Lx = Px = post = 0.0;
                        } else {
                            Lx = MIXED ? s.Lx[c] : (s.Lx[c] + dsd) / 2.0 + lconst;
                            Px = s.Px[c];
                            post = gamma * Lx + Px;
                            ham = post + s.K[c];
                        }
                        double dham = s.ham[c] - ham;
                        if (tuning) score[jj] = s.blown[c] ? 0.0 : s.S[c] * exp(fmin(0.0, dham));
                        double u = rng_uniform(a.seed, stream, P_MH, iter, jj, 0);
                        if (dham > log(u) && !s.blown[c]) {
                            s.acc[c] = 1;
                            s.L[c] = Lx;
                            s.P[c] = Px;
                            s.post[c] = post;
                        }
                        if (!tuning) {
                            Ln[jj] = s.L[c];
                            Pn[jj] = s.P[c];
                        }
                    }
                }
                __syncthreads();
#pragma unroll
                for (int q = 0; q < CT; ++q) {
                    int c = tx * CT + q;
                    if (s.j[c] >= s.jend[c]) continue;
                    bool accd = s.acc[c];
#pragma unroll
                    for (int i = 0; i < RT; ++i) {
                        int r = ty * RT + i;
                        if (accd) xc[i][q] = x[i][q];
                        if (!tuning && r < D) pnew[(size_t)s.j[c] * D + r] = (double)xc[i][q];
                    }
                }
                __syncthreads();
                if (tid < C && s.j[tid] < s.jend[tid]) s.j[tid] += 1;
                __syncthreads();
            }
            if (tuning) {
                // resample the tuned step sizes by score (smc_slip.f90:1098-1207)
                // children in ascending order: mark tuned ones, compact
                for (int q = tid; q < nq; q += NT) {
                    int k = keys[q] & 0xffff;
                    for (int jj = ids[k]; jj < ids[k] + cnt[k]; ++jj) sub[jj] = 1;
                }
                __syncthreads();
                int carry = 0;
                for (int base = 0; base < N; base += NT) {
                    int jj = base + tid;
                    int v = jj < N ? (sub[jj] == 1) : 0, tot;
                    int ex = block_exscan(v, (int *)scr, tot);
                    __syncthreads();
                    if (jj < N) {
                        // reuse keys[] for the compacted child list
                        if (v) keys[carry + ex] = jj;
                        sub[jj] = 0;
                    }
                    carry += tot;
                    __syncthreads();
                }
                const int msub = carry;
                double ps = 0.0;
                for (int q = tid; q < msub; q += NT) ps += score[keys[q]];
                double ssum = block_sum(ps, scr);
                bool degenerate = ssum < 1e-5;
                if (degenerate) ssum = (double)msub;
                __syncthreads();
                for (int q = tid; q < msub; q += NT) w[q] = (degenerate ? 1.0 : score[keys[q]]) / ssum;
                __syncthreads();
                double uh, ul;
                rng_quad_uniform(a.seed, stream, RNG_TUNE_RES, iter, uh, ul);
                long long tot = scan_counts(w, msub, N, uh, ul, sub, (dd *)scr, llscr, &s_tie);
                __syncthreads();
                if (tot == N) {
                    // expand counts into the new step-size list
                    int carry2 = 0;
                    for (int base = 0; base < msub; base += NT) {
                        int q = base + tid;
                        int v = q < msub ? sub[q] : 0, tt;
                        int ex = block_exscan(v, (int *)scr, tt);
                        if (q < msub)
                            for (int r = 0; r < v; ++r) dtn[carry2 + ex + r] = dtau[keys[q]];
                        carry2 += tt;
                        __syncthreads();
                    }
                    for (int k = tid; k < N; k += NT) dtau[k] = dtn[k];
                } else if (tid == 0) {
                    atomicOr(&s_status, SMCGPU_ST_TUNE_COUNT);
                }
                __syncthreads();
                for (int k = tid; k < NP2; k += NT) sub[k] = 0;
                dd pd = {0.0, 0.0};
                for (int k = tid; k < N; k += NT) pd = dd_add_d(pd, dtau[k]);
                dd sm = block_sum_dd(pd, (dd *)scr);
                double mean_hi = sm.hi / N;
                double mean_lo = (fma(-mean_hi, (double)N, sm.hi) + sm.lo) / N;
                double lm = log(mean_hi) + mean_lo / mean_hi;
                log_up = lm + log(5.0);
                log_lo = lm - log(5.0);
                __syncthreads();
            }
        }
        // adopt the new population
        for (size_t e = tid; e < (size_t)N * D; e += NT) parts[e] = pnew[e];
        for (int k = tid; k < N; k += NT) { Lc[k] = Ln[k]; Pc[k] = Pn[k]; }
        __syncthreads();
        ++iter;
    }
    if (tid == 0) {
        int st = s_status;
        if (!isfinite(neglog)) st |= SMCGPU_ST_NONFINITE;
        a.neglog[th] = neglog;
        atomicOr(a.status + th, st);
        a.nstage[th] = iter - 1;
    }
}

template <typename T, int RT, int CT>
static size_t inner_smem_bytes() {
    using TL = Tile<T, RT, CT>;
    constexpr int DP = TL::DP, C = TL::C;
    size_t b = (size_t)2 * DP * DP * sizeof(T) + (size_t)2 * DP * C * sizeof(T);
    b += (size_t)4 * DP * sizeof(T);
    b += (size_t)6 * DP * sizeof(double) + (size_t)TYN * C * sizeof(double) + 64 * sizeof(double);
    b += (size_t)9 * C * sizeof(double) + (size_t)(6 * C + 2) * sizeof(int) + 8 * sizeof(long long) + 64;
    return b;
}

template <typename T, int RT, int CT>
static cudaError_t launch_inner_t(const MeshDev &m, const InnerArgs &a, cudaStream_t s) {
    size_t sm = inner_smem_bytes<T, RT, CT>();
    cudaError_t e = cudaFuncSetAttribute(inner_kernel<T, RT, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    inner_kernel<T, RT, CT><<<a.n_theta, NT, sm, s>>>(m, a);
    return cudaGetLastError();
}

cudaError_t launch_inner(const MeshDev &m, const InnerArgs &a, cudaStream_t s, const char **why) {
    if (a.n_theta <= 0) return cudaSuccess;
    int D = a.D;
    if (a.N > 65535 || a.NP2 > 65536) { *why = "nparticle_slip must be < 65536"; return cudaErrorInvalidValue; }
    if (!a.mixed) {
        if (D <= 32) return launch_inner_t<double, 2, 2>(m, a, s);
        if (D <= 64) return launch_inner_t<double, 4, 2>(m, a, s);
        if (D <= 96) return launch_inner_t<double, 6, 2>(m, a, s);
    } else {
        if (D <= 32) return launch_inner_t<float, 2, 4>(m, a, s);
        if (D <= 64) return launch_inner_t<float, 4, 4>(m, a, s);
        if (D <= 96) return launch_inner_t<float, 6, 4>(m, a, s);
        if (D <= 128) return launch_inner_t<float, 8, 4>(m, a, s);
    }
    *why = "slip dimension too large for the shared-memory inner kernel";
    return cudaErrorInvalidValue;
}

cudaError_t launch_gibbs(const MeshDev &m, const InnerArgs &a, cudaStream_t s) {
    if (a.n_theta <= 0) return cudaSuccess;
    const int wpb = 4;
    size_t sm = (size_t)wpb * 2 * a.D * sizeof(double);
    unsigned blocks = (unsigned)((a.n_theta + wpb - 1) / wpb);
    if (a.mixed) {
        cudaFuncSetAttribute(gibbs_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        gibbs_kernel<true><<<blocks, wpb * 32, sm, s>>>(m, a);
    } else {
        cudaFuncSetAttribute(gibbs_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        gibbs_kernel<false><<<blocks, wpb * 32, sm, s>>>(m, a);
    }
    return cudaGetLastError();
}

}  // namespace smc
