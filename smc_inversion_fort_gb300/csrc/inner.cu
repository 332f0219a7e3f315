// Inner tempered SMC over slip (slip_smc_exec, smc_slip.f90:1445-1663):
// one GROUP of W warps per geometry particle, G = 8/W groups per CTA.
//
// The HMC children of one parent form a Metropolis chain
// (smc_slip.f90:591-730: child k starts where child k-1 stopped), so an
// inner stage is a set of chains of uneven length.  Every warp of a group
// runs C = 8 chain slots in lock step and refills a slot from the group's
// parent queue (sorted by descending child count) when its chain ends.  A
// leapfrog step of a warp's 8 slots is the product grad = M x of the stage
// matrix M = gamma A + L^T L / alpha^2 (shared memory, one copy per group)
// with the warp's DP x 8 slot tile; lane l owns rows (l%16)*RT.. and slots
// (l/16)*4.. and applies the momentum / position update, the reflection into
// [0, max_slip] and the blow-up test to its own entries, so a step needs no
// synchronisation beyond the warp.  The warps of a group meet only at stage
// boundaries (named barrier per group).  W trades per-geometry latency
// (more slots: fewer rounds per stage) against geometries per SM; the host
// picks it from the batch size.  Random draws are addressed by (stage,
// purpose, child index, dimension): the slot schedule does not change results.
//
// FP64 (T = double) follows the reference's algebra in FP64.  MIXED
// (T = float) runs the leapfrog in FP32 about the stage mean sbar with the
// constant part of the gradient and the end-point energies formed in FP64,
// and the tempering bisection in FP32 before one FP64 pass for the weights
// and the evidence increment.
#include <type_traits>

#include "common.cuh"
#include "ddreal.cuh"
#include "inner.h"
#include "q128.cuh"

namespace smc {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int CW = 8;    // chain slots per warp
constexpr int CTW = 4;   // slots per lane
constexpr int RGW = 16;  // row groups per warp

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
template <typename T>
__device__ __forceinline__ void reflect_w(T &x, T &p, T mx, int &flag) {
    int it = 0;
    while (x < T(0) || x > mx) {
        if (x > mx) { x = T(2) * mx - x; p = -p; }
        if (x < T(0)) { x = -x; p = -p; }
        if (++it > 1000000) { flag |= SMCGPU_ST_REFLECT_CAP; break; }
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
        double t = 0.0;
        for (int w = 0; w < W; ++w) t += scr[w];
        return t;
    }
    __device__ double min(double v) const {
        v = wmin(v);
        if (W == 1) return v;
        sync();
        if (lane == 0) scr[wl] = v;
        sync();
        double t = scr[0];
        for (int w = 1; w < W; ++w) t = fmin(t, scr[w]);
        return t;
    }
    __device__ dd sum_dd(dd v) const {
        v = wsum_dd(v);
        if (W == 1) return v;
        dd *s = (dd *)scr;
        sync();
        if (lane == 0) s[wl] = v;
        sync();
        dd t = s[0];
        for (int w = 1; w < W; ++w) t = dd_add(t, s[w]);
        return t;
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

// shared memory of one group
template <typename T, int RT>
struct GroupSmem {
    static constexpr int DP = RGW * RT;
    __host__ __device__ static size_t bytes(int W) {
        return (size_t)DP * DP * sizeof(T) + (size_t)W * 2 * DP * CW * sizeof(T) + (size_t)4 * DP * sizeof(T) +
               (size_t)6 * DP * sizeof(double) + (size_t)W * CW * (5 * sizeof(double) + 5 * sizeof(int)) +
               (size_t)(4 * W + 8) * sizeof(double);
    }
};

}  // namespace

template <typename T, int RT>
__global__ void __launch_bounds__(256) inner_group_kernel(MeshDev m, InnerArgs a, int W, int G) {
    constexpr int DP = RGW * RT;
    constexpr bool MIXED = std::is_same<T, float>::value;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Group grp;
    grp.id = warp / W;
    grp.W = W;
    grp.wl = warp % W;
    grp.lane = lane;
    grp.gt = grp.wl * 32 + lane;
    grp.nt = 32 * W;
    const int th = blockIdx.x * G + grp.id;
    if (grp.id >= G || th >= a.n_theta) return;
    const int N = a.N, D = a.D, NP2 = a.NP2;
    const int rg = lane & 15, cg = lane >> 4, gt = grp.gt, gnt = grp.nt, wl = grp.wl;

    extern __shared__ __align__(16) unsigned char smem_all[];
    unsigned char *smem = smem_all + (size_t)grp.id * GroupSmem<T, RT>::bytes(W);
    T *Msm = (T *)smem;
    T *Xw0 = Msm + DP * DP + (size_t)wl * 2 * DP * CW, *Xw1 = Xw0 + DP * CW;   // this warp's tiles
    T *tcov = Msm + DP * DP + (size_t)W * 2 * DP * CW, *tmean = tcov + DP, *tcv = tmean + DP, *tisc = tcv + DP;
    double *vb = (double *)(tisc + DP);
    double *vcov = vb + DP, *vmean = vcov + DP, *vg = vmean + DP, *vh = vg + DP, *vc = vh + DP;
    double *sdall = vc + DP;                                   // W * 5 * CW doubles
    double *sd = sdall + (size_t)wl * 5 * CW;
    double *sL = sd, *sP = sd + CW, *spost = sd + 2 * CW, *sham = sd + 3 * CW, *sdt = sd + 4 * CW;
    int *siall = (int *)(sdall + (size_t)W * 5 * CW);        // W * 5 * CW ints
    int *si = siall + (size_t)wl * 5 * CW;
    int *spar = si, *sj = si + CW, *sjend = si + 2 * CW, *sfresh = si + 3 * CW, *sblown = si + 4 * CW;
    double *gscr = (double *)(siall + (size_t)W * 5 * CW + ((W * 5 * CW) & 1));
    int *gint = (int *)(gscr + 4 * W);                          // [0] queue head, [1] queue length, [2] status
    grp.scr = gscr;

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

    if (gt == 0) gint[2] = 0;
    for (int i = gt; i < DP; i += gnt) vb[i] = i < D ? bth[i] : 0.0;
    for (int k = gt; k < N; k += gnt) dtau[k] = exp(-5.0);
    if (MIXED)
        for (int e = gt; e < D * D; e += gnt) A32[e] = (float)Ath[e];
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

    double gamma = 0.0, neglog = 0.0, log_up = 0.0, log_lo = -1e1;
    int iter = 1;
    while (1.0 - gamma > 10e-8) {
        // ---- next tempering exponent (smc_slip.f90:314-387)
        double lmin = 1e300;
        for (int k = gt; k < N; k += gnt) lmin = fmin(lmin, Lc[k]);
        lmin = grp.min(lmin);
        const double gprev = gamma;
        double lower = gprev, upper = 1.0, err = 1.0, g = 1.0;
        int bcnt = 0;
        const double tol = MIXED ? 1e-6 : 1e-10;
        while (err > tol) {
            g = (lower + upper) / 2.0;
            double dg = g - gprev, cv;
            if (MIXED) {
                float dgf = (float)dg;
                double ps = 0.0, ps2 = 0.0;
                for (int k = gt; k < N; k += gnt) {
                    float wk = expf(-dgf * (float)(Lc[k] - lmin));
                    ps += wk;
                    ps2 += (double)wk * wk;
                }
                double s1 = grp.sum(ps), s2 = grp.sum(ps2);
                double mean = s1 / N;
                cv = sqrt(fmax(s2 / N - mean * mean, 0.0)) / mean;
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
            for (int k = gt; k < N; k += gnt) w[k] = dd_div_into_w(w[k], sw);
            grp.sync();
        }
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
        // ---- stage matrix and centring terms
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
        }
        grp.sync();

        // ---- HMC passes: tuning (every tf-th parent, smc_slip.f90:919-1214),
        // then sampling (smc_slip.f90:591-730)
        for (int pass = 0; pass < 2; ++pass) {
            const bool tuning = pass == 0;
            const uint32_t P_MOM = tuning ? RNG_TUNE_MOM : RNG_SMP_MOM;
            const uint32_t P_MH = tuning ? RNG_TUNE_MH : RNG_SMP_MH;
            double nql = 0.0;
            for (int k = gt; k < NP2; k += gnt) {
                bool ok = k < N && cnt[k] > 0 && (!tuning || k % a.tf == 0);
                keys[k] = ok ? (int)(((unsigned)(N - cnt[k]) << 16) | (unsigned)k) : 0x7fffffff;
                nql += ok;
            }
            const int nq = (int)grp.sum(nql);
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
            if (gt == 0) gint[0] = 0;
            if (lane < CW) { sj[lane] = 0; sjend[lane] = 0; spar[lane] = -1; }
            grp.sync();
            T xc[RT][CTW], x[RT][CTW], p[RT][CTW], acc[RT][CTW];
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
                                if (fabs(x[i][q]) > T(1e3)) atomicOr(&sblown[c], 1);
                                else reflect_w<T>(x[i][q], p[i][q], mx, flag);
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
        for (size_t e = gt; e < (size_t)N * D; e += gnt) parts[e] = pnew[e];
        for (int k = gt; k < N; k += gnt) { Lc[k] = Ln[k]; Pc[k] = Pn[k]; }
        grp.sync();
        ++iter;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) status |= __shfl_xor_sync(FULL, status, o);
    if (lane == 0 && status) atomicOr(&gint[2], status);
    grp.sync();
    if (gt == 0) {
        int st = gint[2];
        if (!isfinite(neglog)) st |= SMCGPU_ST_NONFINITE;
        a.neglog[th] = neglog;
        atomicOr(a.status + th, st);
        a.nstage[th] = iter - 1;
    }
}

template <typename T, int RT>
static cudaError_t launch_group_t(const MeshDev &m, const InnerArgs &a, cudaStream_t s, int W) {
    int dev = 0, maxsm = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (W <= 0) {
        // warps per geometry from the batch size: enough geometries in flight
        // to fill every SM with 8 warps, otherwise more slots per geometry
        const long long slots = 8LL * nsm;
        W = 1;
        while (W < 8 && (long long)a.n_theta * W * 2 <= slots) W *= 2;
    }
    size_t per = GroupSmem<T, RT>::bytes(W);
    int G = (int)std::min<size_t>((size_t)(8 / W), (size_t)maxsm / per);
    while (G < 1 && W > 1) {
        W /= 2;
        per = GroupSmem<T, RT>::bytes(W);
        G = (int)std::min<size_t>((size_t)(8 / W), (size_t)maxsm / per);
    }
    if (G < 1) return cudaErrorInvalidValue;
    size_t sm = per * G;
    cudaError_t e = cudaFuncSetAttribute(inner_group_kernel<T, RT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    unsigned blocks = (unsigned)((a.n_theta + G - 1) / G);
    inner_group_kernel<T, RT><<<blocks, 32 * W * G, sm, s>>>(m, a, W, G);
    return cudaGetLastError();
}

cudaError_t launch_inner(const MeshDev &m, const InnerArgs &a, cudaStream_t s, const char **why) {
    if (a.n_theta <= 0) return cudaSuccess;
    if (a.N > 32767) { *why = "nparticle_slip must be < 32768"; return cudaErrorInvalidValue; }
    const int D = a.D;
    const int W = a.warps_per_theta;
    if (!a.mixed) {
        if (D <= 32) return launch_group_t<double, 2>(m, a, s, W);
        if (D <= 64) return launch_group_t<double, 4>(m, a, s, W);
        if (D <= 96) return launch_group_t<double, 6>(m, a, s, W);
        if (D <= 128) return launch_group_t<double, 8>(m, a, s, W);
    } else {
        if (D <= 32) return launch_group_t<float, 2>(m, a, s, W);
        if (D <= 64) return launch_group_t<float, 4>(m, a, s, W);
        if (D <= 96) return launch_group_t<float, 6>(m, a, s, W);
        if (D <= 128) return launch_group_t<float, 8>(m, a, s, W);
        if (D <= 192) return launch_group_t<float, 12>(m, a, s, W);
    }
    *why = "slip dimension too large for the shared-memory inner kernel";
    return cudaErrorInvalidValue;
}

}  // namespace smc
