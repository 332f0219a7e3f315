// C ABI entry points of the nested likelihood (fault_calc_likelihood), the
// outer SMC (fault_smc_exec) and the stand-alone resampling primitive.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "context.h"
#include "inner.h"

#define CU(call, where)                                          \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ctx->cuda_fail(e_, where); \
    } while (0)

namespace {

// NVTX range over a scope (header-only NVTX v3: inert unless a profiler or
// tracer is attached), named for the stage of the path it covers
struct Range {
    explicit Range(const std::string &name) { nvtxRangePushA(name.c_str()); }
    ~Range() { nvtxRangePop(); }
};

struct NestedOpts {
    double *trace_gamma = nullptr, *trace_inc = nullptr;  // device, [n][max_stages+2]
    int *nstage = nullptr;                                // device [n]
    double *particles_out = nullptr;                      // host [N][D] of theta 0 (single-theta call)
    double *lik_out = nullptr, *prior_out = nullptr;      // host [N]
    double *mean_dev = nullptr;                           // device [n][D]: mean final inner population
    // when set and the batch fits one chunk: stop before the inner SMC launch
    // and return its arguments here (*deferred = true); the caller launches it
    smc::InnerArgs *defer = nullptr;
    bool *deferred = nullptr;
};

int next_pow2(int n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

}  // namespace

// The step engine and warps per geometry of this context's batches: the
// configured engine, or under SMCGPU_ENGINE_AUTO the engine table's entry for
// the slip dimension (default: warp MMA / CUDA cores up to their limits, the
// global-matrix engine above).
void smc_resolve_engine(const smcgpu_ctx *ctx, int *engine, int *warps) {
    *engine = ctx->cfg.inner_engine;
    *warps = ctx->cfg.inner_warps;
    if (*engine != SMCGPU_ENGINE_AUTO) return;
    const int D = ctx->mesh.D, pi = ctx->cfg.precision == SMCGPU_PREC_MIXED ? 1 : 0;
    const std::vector<int> &dm = ctx->eng_dmax[pi];
    for (size_t k = 0; k < dm.size(); ++k)
        if (D <= dm[k]) {
            *engine = ctx->eng_engine[pi][k];
            *warps = ctx->eng_warps[pi][k];
            return;
        }
    *engine = pi ? (D <= 256 ? SMCGPU_ENGINE_MMA : SMCGPU_ENGINE_GLOBAL)
                 : (D <= 128 ? SMCGPU_ENGINE_CUDA : SMCGPU_ENGINE_GLOBAL);
    *warps = 0;
}

namespace {

// streamed stage matrix of the warp-MMA inner engine: uint4 per geometry (0 when unused)
size_t afrag_per_theta(const smcgpu_ctx *ctx) {
    const int D = ctx->mesh.D;
    int engine, warps;
    smc_resolve_engine(ctx, &engine, &warps);
    const bool streamed = ctx->cfg.precision == SMCGPU_PREC_MIXED && engine == SMCGPU_ENGINE_MMA &&
                          D > 128 && D <= 256;
    return streamed ? (size_t)256 * 256 / 4 : 0;
}

// global-matrix engine: bytes per geometry of the stage matrix and of the
// slots' chain states (0 when another engine runs the batch)
size_t gl_bytes_per_theta(const smcgpu_ctx *ctx, size_t *mgl, size_t *glxc) {
    const int D = ctx->mesh.D;
    const bool mixed = ctx->cfg.precision == SMCGPU_PREC_MIXED;
    const size_t el = mixed ? sizeof(float) : sizeof(double);
    int engine, warps;
    smc_resolve_engine(ctx, &engine, &warps);
    const bool on = smc::inner_uses_global(mixed, engine, D);
    *mgl = on ? (size_t)D * D * el : 0;
    *glxc = on ? (size_t)16 * D * el : 0;
    return *mgl + *glxc;
}

size_t bytes_per_theta(const smcgpu_ctx *ctx) {
    const smc::MeshPattern &p = ctx->mesh;
    size_t D = p.D, N = ctx->cfg.nparticle_slip, NP2 = next_pow2((int)N);
    size_t b = D * ctx->nobs * 8 + D * std::max(ctx->nsar, 0) * 8 + D * D * 12 + D * 8 + 8;
    b += (size_t)p.nrow * 9 * 8 + D * 9 * 8 + p.ll_col.size() * 8 + sizeof(smc::ThetaAux);
    b += 2 * N * D * 8 + 9 * N * 8 + 4 * NP2 * 4 + p.nplane * sizeof(smc::PlaneGeom) + 64;
    b += afrag_per_theta(ctx) * sizeof(uint4);
    size_t m1, m2;
    b += gl_bytes_per_theta(ctx, &m1, &m2);
    return b;
}

// Run statistics: an event recorded on the stream, kept for later timing.
cudaError_t stats_mark(std::vector<cudaEvent_t> &v, cudaStream_t s) {
    cudaEvent_t e = nullptr;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    v.push_back(e);
    return cudaEventRecord(e, s);
}

// Sums the (start, stop) pairs of v into ms and releases the events.
cudaError_t stats_resolve(std::vector<cudaEvent_t> &v, double &ms) {
    cudaError_t r = cudaSuccess;
    for (size_t i = 0; i + 1 < v.size(); i += 2) {
        float t = 0.0f;
        if (r == cudaSuccess) r = cudaEventSynchronize(v[i + 1]);
        if (r == cudaSuccess) r = cudaEventElapsedTime(&t, v[i], v[i + 1]);
        ms += t;
    }
    for (cudaEvent_t e : v) cudaEventDestroy(e);
    v.clear();
    return r;
}

// Runs the nested evaluation for n thetas already on the device, in chunks.
int nested_batch(smcgpu_ctx *ctx, int n, const double *theta_dev, uint64_t seed, const unsigned long long *streams_dev,
                 double *neglog_dev, int *status_dev, const NestedOpts &opt) {
    const smc::MeshPattern &pm = ctx->mesh;
    const int D = pm.D, N = ctx->cfg.nparticle_slip, NP2 = next_pow2(N), nd = pm.ndim_fault;
    cudaStream_t s = ctx->stream;
    if (const char *why = smc::inner_size_limit(ctx->cfg.precision == SMCGPU_PREC_MIXED, ctx->cfg.inner_engine, D, N))
        return ctx->fail(SMCGPU_ERR_ARG, why);
    Range range("nested batch: " + std::to_string(n) + " geometries, D = " + std::to_string(D));
    size_t per = bytes_per_theta(ctx);
    size_t budget = (size_t)48 << 30;
    size_t freeb = 0, totb = 0;
    if (cudaMemGetInfo(&freeb, &totb) == cudaSuccess) budget = std::min(budget, freeb / 2);
    int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)n, budget / per));
    CU(ctx->d_planes.ensure((size_t)chunk * pm.nplane), "alloc");
    CU(ctx->d_gmat.ensure((size_t)chunk * D * ctx->nobs), "alloc gmat");
    CU(ctx->d_gw.ensure((size_t)chunk * D * std::max(ctx->nsar, 1)), "alloc gw");
    CU(ctx->d_A.ensure((size_t)chunk * D * D), "alloc A");
    CU(ctx->d_b.ensure((size_t)chunk * D), "alloc b");
    CU(ctx->d_dsd.ensure((size_t)chunk), "alloc dsd");
    CU(ctx->d_lval.ensure((size_t)chunk * pm.nrow * 9), "alloc lval");
    CU(ctx->d_ltval.ensure((size_t)chunk * D * 9), "alloc ltval");
    CU(ctx->d_llval.ensure((size_t)chunk * std::max<size_t>(pm.ll_col.size(), 1)), "alloc llval");
    CU(ctx->d_aux.ensure((size_t)chunk), "alloc aux");
    CU(ctx->d_parts.ensure((size_t)chunk * N * D), "alloc particles");
    CU(ctx->d_parts_new.ensure((size_t)chunk * N * D), "alloc particles");
    CU(ctx->d_dbuf.ensure((size_t)chunk * 9 * N), "alloc dbuf");
    CU(ctx->d_ibuf.ensure((size_t)chunk * 4 * NP2), "alloc ibuf");
    CU(ctx->d_A32.ensure((size_t)chunk * D * D), "alloc A32");
    CU(ctx->d_lv32.ensure((size_t)chunk * std::max(pm.nrow, 1) * 9), "alloc lv32");
    CU(ctx->d_ll32.ensure((size_t)chunk * std::max<size_t>(pm.ll_col.size(), 1)), "alloc ll32");
    if (afrag_per_theta(ctx)) CU(ctx->d_afrag.ensure((size_t)chunk * afrag_per_theta(ctx)), "alloc stage matrices");
    size_t mgl_b = 0, glxc_b = 0;
    if (gl_bytes_per_theta(ctx, &mgl_b, &glxc_b)) {
        CU(ctx->d_mgl.ensure((size_t)chunk * mgl_b), "alloc global stage matrices");
        CU(ctx->d_glxc.ensure((size_t)chunk * glxc_b), "alloc chain states");
    }
    CU(ctx->d_nstage_tmp.ensure((size_t)chunk), "alloc");
    auto &stats = ctx->stats;
    if (stats.on && stats.inner_ev.size() > 4096) {
        CU(stats_resolve(stats.inner_ev, stats.inner_ms), "stats");
        CU(stats_resolve(stats.batch_ev, stats.batch_ms), "stats");
    }
    for (int t0 = 0; t0 < n; t0 += chunk) {
        int nb = std::min(chunk, n - t0);
        const double *th = theta_dev + (size_t)t0 * nd;
        if (stats.on) {
            CU(stats_mark(stats.batch_ev, s), "stats event");
            stats.evals += nb;
        }
        CU(smc::launch_planes(ctx->md, nb, th, ctx->d_planes.p, s), "planes kernel");
        CU(smc::launch_greens(ctx->md, nb, ctx->d_planes.p, SMCGPU_PREC_FP64, ctx->d_gmat.p, s), "greens kernel");
        CU(smc::launch_setup(ctx->md, nb, th, ctx->d_planes.p, ctx->d_lval.p, ctx->d_ltval.p, ctx->d_llval.p,
                             ctx->d_aux.p, s), "setup kernel");
        CU(smc::launch_gram(ctx->md, nb, ctx->d_gmat.p, ctx->obs_roww(), ctx->obs_dx(), ctx->d_aux.p, ctx->dsd_sar,
                            ctx->dsd_gnss, ctx->d_A.p, ctx->d_b.p, ctx->d_dsd.p, ctx->d_gw.p, s), "gram kernel");
        CU(cudaMemsetAsync(status_dev + t0, 0, (size_t)nb * sizeof(int), s), "memset");
        CU(cudaMemsetAsync(ctx->d_ibuf.p, 0, (size_t)nb * 4 * NP2 * sizeof(int), s), "memset");
        smc::InnerArgs a{};
        a.n_theta = nb; a.N = N; a.NP2 = NP2; a.D = D;
        a.mixed = ctx->cfg.precision == SMCGPU_PREC_MIXED;
        a.ntau = ctx->cfg.ntau; a.tf = ctx->cfg.tuning_factor; a.max_stages = ctx->cfg.max_stages;
        a.cv = ctx->cfg.cv_inner; a.max_slip = ctx->cfg.max_slip; a.seed = seed;
        a.streams = streams_dev + t0;
        a.A = ctx->d_A.p; a.b = ctx->d_b.p; a.dsd = ctx->d_dsd.p; a.lval = ctx->d_lval.p; a.llval = ctx->d_llval.p;
        a.aux = ctx->d_aux.p;
        a.parts = ctx->d_parts.p; a.parts_new = ctx->d_parts_new.p; a.dbuf = ctx->d_dbuf.p; a.ibuf = ctx->d_ibuf.p;
        a.neglog = neglog_dev + t0; a.status = status_dev + t0;
        a.nstage = opt.nstage ? opt.nstage + t0 : ctx->d_nstage_tmp.p;
        a.trace_gamma = opt.trace_gamma ? opt.trace_gamma + (size_t)t0 * (a.max_stages + 2) : nullptr;
        a.trace_inc = opt.trace_inc ? opt.trace_inc + (size_t)t0 * (a.max_stages + 2) : nullptr;
        CU(smc::launch_gibbs(ctx->md, a, s), "gibbs kernel");
        const char *why = nullptr;
        a.A32 = ctx->d_A32.p;
        a.lv32 = ctx->d_lv32.p;
        a.ll32 = ctx->d_ll32.p;
        a.afrag = afrag_per_theta(ctx) ? ctx->d_afrag.p : nullptr;
        a.mgl = mgl_b ? (void *)ctx->d_mgl.p : nullptr;
        a.glxc = glxc_b ? (void *)ctx->d_glxc.p : nullptr;
        CU(ctx->d_queue.ensure(1), "alloc queue");
        a.queue = ctx->d_queue.p;
        smc_resolve_engine(ctx, &a.engine, &a.warps_per_theta);
        a.counters = stats.on ? stats.d_counters.p : nullptr;
        if (ctx->parent && ctx->parent->stats.on) a.counters = ctx->parent->stats.d_counters.p;
        if (opt.defer && nb == n && !opt.mean_dev && !opt.particles_out && !stats.on) {
            *opt.defer = a;
            *opt.deferred = true;
            return SMCGPU_OK;
        }
        if (stats.on) CU(stats_mark(stats.inner_ev, s), "stats event");
        cudaError_t e = smc::launch_inner(ctx->md, a, s, &why);
        if (e != cudaSuccess) {
            if (why) return ctx->fail(SMCGPU_ERR_ARG, why);
            return ctx->cuda_fail(e, "inner kernel");
        }
        if (stats.on) CU(stats_mark(stats.inner_ev, s), "stats event");
        if (opt.mean_dev)
            CU(smc::launch_mean_particles(nb, N, D, ctx->d_parts.p, opt.mean_dev + (size_t)t0 * D, s), "mean kernel");
        if (opt.particles_out && t0 == 0) {
            CU(cudaMemcpyAsync(opt.particles_out, ctx->d_parts.p, (size_t)N * D * sizeof(double),
                               cudaMemcpyDeviceToHost, s), "copy particles");
            CU(cudaMemcpyAsync(opt.lik_out, ctx->d_dbuf.p, (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, s),
               "copy");
            CU(cudaMemcpyAsync(opt.prior_out, ctx->d_dbuf.p + N, (size_t)N * sizeof(double), cudaMemcpyDeviceToHost,
                               s), "copy");
        }
        if (stats.on) CU(stats_mark(stats.batch_ev, s), "stats event");
    }
    return SMCGPU_OK;
}

// G, then the Gram products, for n thetas already on the device, in chunks;
// the products are copied to the host buffers after each chunk
int gram_batch(smcgpu_ctx *ctx, int n, const double *theta_dev, double *gsg, double *gsd, double *dsd) {
    const smc::MeshPattern &pm = ctx->mesh;
    const int D = pm.D, nd = pm.ndim_fault;
    cudaStream_t s = ctx->stream;
    const size_t per = (size_t)D * ctx->nobs * 8 + (size_t)D * std::max(ctx->nsar, 0) * 8 + (size_t)D * D * 8 +
                       (size_t)D * 8 + (size_t)pm.nrow * 9 * 8 + (size_t)D * 9 * 8 + pm.ll_col.size() * 8 + 256;
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)n, ((size_t)4 << 30) / per));
    CU(ctx->d_planes.ensure((size_t)chunk * pm.nplane), "alloc");
    CU(ctx->d_gmat.ensure((size_t)chunk * D * ctx->nobs), "alloc gmat");
    CU(ctx->d_gw.ensure((size_t)chunk * D * std::max(ctx->nsar, 1)), "alloc gw");
    CU(ctx->d_A.ensure((size_t)chunk * D * D), "alloc A");
    CU(ctx->d_b.ensure((size_t)chunk * D), "alloc b");
    CU(ctx->d_dsd.ensure((size_t)chunk), "alloc dsd");
    CU(ctx->d_lval.ensure((size_t)chunk * pm.nrow * 9), "alloc lval");
    CU(ctx->d_ltval.ensure((size_t)chunk * D * 9), "alloc ltval");
    CU(ctx->d_llval.ensure((size_t)chunk * std::max<size_t>(pm.ll_col.size(), 1)), "alloc llval");
    CU(ctx->d_aux.ensure((size_t)chunk), "alloc aux");
    for (int t0 = 0; t0 < n; t0 += chunk) {
        const int nb = std::min(chunk, n - t0);
        const double *th = theta_dev + (size_t)t0 * nd;
        CU(smc::launch_planes(ctx->md, nb, th, ctx->d_planes.p, s), "planes kernel");
        CU(smc::launch_greens(ctx->md, nb, ctx->d_planes.p, SMCGPU_PREC_FP64, ctx->d_gmat.p, s), "greens kernel");
        CU(smc::launch_setup(ctx->md, nb, th, ctx->d_planes.p, ctx->d_lval.p, ctx->d_ltval.p, ctx->d_llval.p,
                             ctx->d_aux.p, s), "setup kernel");
        CU(smc::launch_gram(ctx->md, nb, ctx->d_gmat.p, ctx->obs_roww(), ctx->obs_dx(), ctx->d_aux.p, ctx->dsd_sar,
                            ctx->dsd_gnss, ctx->d_A.p, ctx->d_b.p, ctx->d_dsd.p, ctx->d_gw.p, s), "gram kernel");
        CU(cudaMemcpyAsync(gsg + (size_t)t0 * D * D, ctx->d_A.p, (size_t)nb * D * D * sizeof(double),
                           cudaMemcpyDeviceToHost, s), "copy gsgmat");
        CU(cudaMemcpyAsync(gsd + (size_t)t0 * D, ctx->d_b.p, (size_t)nb * D * sizeof(double), cudaMemcpyDeviceToHost,
                           s), "copy gsdvec");
        CU(cudaMemcpyAsync(dsd + t0, ctx->d_dsd.p, (size_t)nb * sizeof(double), cudaMemcpyDeviceToHost, s), "copy dsd");
        CU(cudaStreamSynchronize(s), "sync");
    }
    return SMCGPU_OK;
}

// Per-geometry meshes (cfg.patch_km > 0): the patch counts of a rectangle
// geometry, nxi = round(length / patch_km), neta = round(width / patch_km),
// clamped to [2, nxi[0]] and [2, neta[0]] (a non-finite size gives 2).
void mesh_of(const smcgpu_ctx *ctx, const double *th, int *nx, int *ne) {
    const double ps = ctx->cfg.patch_km;
    auto count = [&](double len, int mx) {
        if (!(len > 0.0) || !std::isfinite(len)) return 2;
        const double v = std::floor(len / ps + 0.5);
        return (int)std::min<double>(std::max<double>(v, 2.0), (double)mx);
    };
    *nx = count(th[3], ctx->cfg.nxi[0]);
    *ne = count(th[4], ctx->cfg.neta[0]);
}

// Nested evaluations of host geometries under per-geometry meshes: the batch
// is split by mesh, each part runs the usual device pipeline in its mesh's
// child context on that context's own stream (all parts launched before any
// is waited for, costliest first), and the results return in the caller's
// order.
int uneven_eval(smcgpu_ctx *ctx, int n, const double *theta, uint64_t seed, const unsigned long long *streams,
                double *neglog, int32_t *status, int32_t *nstage, double *tg, double *ti) {
    const int nd = ctx->mesh.ndim_fault, ms = ctx->cfg.max_stages + 2;
    Range range("per-geometry meshes: " + std::to_string(n) + " geometries");
    struct Part {
        int nx = 0, ne = 0;
        std::vector<int> idx;
        std::vector<double> th;
        std::vector<unsigned long long> sid;
        smcgpu_ctx *ch = nullptr;
        smc::InnerArgs args{};        // the deferred inner launch of this part
        bool deferred = false;
        cudaEvent_t ready = nullptr;  // set-up done (then: inner SMC done)
        Part() = default;
        Part(const Part &) = delete;
        Part &operator=(const Part &) = delete;
        ~Part() {
            if (ready) cudaEventDestroy(ready);
        }
    };
    std::map<long long, Part> parts;
    for (int i = 0; i < n; ++i) {
        int nx, ne;
        mesh_of(ctx, theta + (size_t)i * nd, &nx, &ne);
        Part &p = parts[(long long)nx * 4096 + ne];
        p.nx = nx;
        p.ne = ne;
        p.idx.push_back(i);
    }
    std::vector<Part *> order;
    for (auto &kv : parts) order.push_back(&kv.second);
    // costliest first: the inner step cost grows as D^2, D = 2 nx ne
    std::stable_sort(order.begin(), order.end(), [](const Part *a, const Part *b) {
        const double ca = (double)a->nx * a->ne * a->nx * a->ne * a->idx.size();
        const double cb = (double)b->nx * b->ne * b->nx * b->ne * b->idx.size();
        return ca > cb;
    });
    const bool want_ns = nstage || tg || ti, want_tr = tg || ti;
    for (Part *p : order) {
        int r = smc_child_context(ctx, p->nx, p->ne, &p->ch);
        if (r) return r;
        smcgpu_ctx *ch = p->ch;
        const int ng = (int)p->idx.size();
        p->th.resize((size_t)ng * nd);
        p->sid.resize(ng);
        for (int q = 0; q < ng; ++q) {
            std::memcpy(&p->th[(size_t)q * nd], theta + (size_t)p->idx[q] * nd, nd * sizeof(double));
            p->sid[q] = streams[p->idx[q]];
        }
        cudaStream_t cs = ch->stream;
        CU(ch->d_theta.upload(p->th.data(), p->th.size(), cs), "upload theta");
        CU(ch->d_streams.upload(p->sid.data(), ng, cs), "upload streams");
        CU(ch->d_neglog.ensure(ng), "alloc");
        CU(ch->d_status.ensure(ng), "alloc");
        NestedOpts opt;
        if (want_ns) {
            CU(ch->d_nstage.ensure(ng), "alloc");
            opt.nstage = ch->d_nstage.p;
        }
        if (want_tr) {
            CU(ch->d_trace.ensure((size_t)2 * ng * ms), "alloc");
            CU(cudaMemsetAsync(ch->d_trace.p, 0, (size_t)2 * ng * ms * sizeof(double), cs), "memset");
            opt.trace_gamma = ch->d_trace.p;
            opt.trace_inc = ch->d_trace.p + (size_t)ng * ms;
        }
        opt.defer = &p->args;
        opt.deferred = &p->deferred;
        r = nested_batch(ch, ng, ch->d_theta.p, seed, ch->d_streams.p, ch->d_neglog.p, ch->d_status.p, opt);
        if (r) return ctx->fail(r, ch->err);
        if (p->deferred) {
            if (!p->ready) CU(cudaEventCreateWithFlags(&p->ready, cudaEventDisableTiming), "event");
            CU(cudaEventRecord(p->ready, cs), "event");
        }
    }
    // The inner SMC of the deferred parts: parts that run on the same kernel
    // instantiation (engine, row tile, warps) share one persistent launch, so
    // the geometries of all their meshes fill the GPU together instead of
    // one small launch per mesh.  A launch runs on its first part's stream
    // after every part's set-up, and every part's stream waits for it.
    {
        std::map<long long, std::vector<Part *>> groups;
        for (Part *p : order)
            if (p->deferred) {
                const smc::InnerArgs &a = p->args;
                groups[smc::inner_launch_key(a.mixed, a.engine, a.D, a.warps_per_theta, n)].push_back(p);
            }
        for (auto &kv : groups) {
            std::vector<Part *> &g = kv.second;
            for (size_t g0 = 0; g0 < g.size(); g0 += smc::INNER_MAX_PARTS) {
                const size_t g1 = std::min(g.size(), g0 + (size_t)smc::INNER_MAX_PARTS);
                cudaStream_t ls = g[g0]->ch->stream;
                static thread_local smc::InnerParts P;   // about 21 KB: kept off the stack
                P.n = (int)(g1 - g0);
                P.start[0] = 0;
                for (size_t q = g0; q < g1; ++q) {
                    Part *p = g[q];
                    const int k = (int)(q - g0);
                    P.m[k] = p->ch->md;
                    P.a[k] = p->args;
                    P.start[k + 1] = P.start[k] + p->args.n_theta;
                    if (p->ch->stream != ls) CU(cudaStreamWaitEvent(ls, p->ready, 0), "wait");
                }
                const char *why = nullptr;
                cudaError_t e = smc::launch_inner_parts(P, ls, &why);
                if (e != cudaSuccess) {
                    if (why) return ctx->fail(SMCGPU_ERR_ARG, why);
                    return ctx->cuda_fail(e, "inner kernel");
                }
                Part *lead = g[g0];
                CU(cudaEventRecord(lead->ready, ls), "event");
                for (size_t q = g0 + 1; q < g1; ++q) CU(cudaStreamWaitEvent(g[q]->ch->stream, lead->ready, 0), "wait");
            }
        }
    }
    std::vector<double> nl, tr;
    std::vector<int32_t> st, ns;
    for (Part *p : order) {
        smcgpu_ctx *ch = p->ch;
        const int ng = (int)p->idx.size();
        CU(cudaStreamSynchronize(ch->stream), "sync");
        nl.resize(ng);
        st.resize(ng);
        CU(cudaMemcpy(nl.data(), ch->d_neglog.p, ng * sizeof(double), cudaMemcpyDeviceToHost), "copy");
        CU(cudaMemcpy(st.data(), ch->d_status.p, ng * sizeof(int32_t), cudaMemcpyDeviceToHost), "copy");
        if (want_ns) {
            ns.resize(ng);
            CU(cudaMemcpy(ns.data(), ch->d_nstage.p, ng * sizeof(int32_t), cudaMemcpyDeviceToHost), "copy");
        }
        if (want_tr) {
            tr.resize((size_t)2 * ng * ms);
            CU(cudaMemcpy(tr.data(), ch->d_trace.p, tr.size() * sizeof(double), cudaMemcpyDeviceToHost), "copy");
        }
        for (int q = 0; q < ng; ++q) {
            const int i = p->idx[q];
            neglog[i] = nl[q];
            status[i] = st[q];
            if (nstage) nstage[i] = ns[q];
            if (tg) std::memcpy(tg + (size_t)i * ms, &tr[(size_t)q * ms], ms * sizeof(double));
            if (ti) std::memcpy(ti + (size_t)i * ms, &tr[(size_t)(ng + q) * ms], ms * sizeof(double));
        }
    }
    if (ctx->stats.on) ctx->stats.evals += n;
    return SMCGPU_OK;
}

int check_ready(smcgpu_ctx *ctx) {
    if (!ctx->has_data) return ctx->fail(SMCGPU_ERR_NODATA, "set_data not called");
    if (ctx->cfg.precision != SMCGPU_PREC_FP64 && ctx->cfg.precision != SMCGPU_PREC_MIXED)
        return ctx->fail(SMCGPU_ERR_ARG, "nested evaluation needs precision FP64 or MIXED");
    return SMCGPU_OK;
}

}  // namespace

extern "C" int32_t smcgpu_gram_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, double *gsgmat,
                                     double *gsdvec, double *dsd) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!ctx->has_data) return ctx->fail(SMCGPU_ERR_NODATA, "gram: set_data not called");
    if (n_theta < 0 || (n_theta > 0 && (!theta || !gsgmat || !gsdvec || !dsd)))
        return ctx->fail(SMCGPU_ERR_ARG, "gram: bad arguments");
    if (n_theta == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    CU(ctx->d_theta.upload(theta, (size_t)n_theta * ctx->mesh.ndim_fault, ctx->stream), "upload theta");
    return gram_batch(ctx, n_theta, ctx->d_theta.p, gsgmat, gsdvec, dsd);
}

extern "C" int32_t smcgpu_resample_counts(smcgpu_ctx *ctx, const double *weights, int32_t n, double u0_hi,
                                          double u0_lo, int32_t *counts) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (n < 0 || (n > 0 && (!weights || !counts))) return ctx->fail(SMCGPU_ERR_ARG, "resample: bad arguments");
    if (n == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    CU(ctx->d_w.upload(weights, n, ctx->stream), "upload weights");
    CU(ctx->d_counts.ensure(n), "alloc counts");
    CU(ctx->d_flag.ensure(1), "alloc flag");
    CU(smc::launch_resample_counts(ctx->d_w.p, n, u0_hi, u0_lo, ctx->d_counts.p, ctx->d_flag.p, ctx->stream),
       "resample kernel");
    CU(cudaMemcpyAsync(counts, ctx->d_counts.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
       "copy counts");
    CU(cudaStreamSynchronize(ctx->stream), "sync");
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_fault_likelihood_batch_dev(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                                     uint64_t seed, const uint64_t *streams_dev, double *neglog_dev,
                                                     int32_t *status_dev) {
    if (!ctx) return SMCGPU_ERR_ARG;
    int r = check_ready(ctx);
    if (r) return r;
    if (n_theta < 0 || (n_theta > 0 && (!theta_dev || !streams_dev || !neglog_dev || !status_dev)))
        return ctx->fail(SMCGPU_ERR_ARG, "fault_likelihood: bad arguments");
    if (n_theta == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    if (ctx->cfg.patch_km > 0.0) {
        // per-geometry meshes: the split by mesh is made on the host
        const int nd = ctx->mesh.ndim_fault;
        std::vector<double> th((size_t)n_theta * nd), nl(n_theta);
        std::vector<unsigned long long> sid(n_theta);
        std::vector<int32_t> st(n_theta);
        CU(cudaMemcpyAsync(th.data(), theta_dev, th.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "copy theta");
        CU(cudaMemcpyAsync(sid.data(), streams_dev, sid.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                           ctx->stream), "copy streams");
        CU(cudaStreamSynchronize(ctx->stream), "sync");
        int r = uneven_eval(ctx, n_theta, th.data(), seed, sid.data(), nl.data(), st.data(), nullptr, nullptr,
                            nullptr);
        if (r) return r;
        CU(cudaMemcpyAsync(neglog_dev, nl.data(), nl.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
           "copy");
        CU(cudaMemcpyAsync(status_dev, st.data(), st.size() * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream),
           "copy");
        CU(cudaStreamSynchronize(ctx->stream), "sync");
        return SMCGPU_OK;
    }
    return nested_batch(ctx, n_theta, theta_dev, seed, (const unsigned long long *)streams_dev, neglog_dev,
                        status_dev, NestedOpts());
}

static int likelihood_host(smcgpu_ctx *ctx, int n, const double *theta, uint64_t seed, const uint64_t *streams,
                           double *neglog_out, int32_t *status_out, int32_t *nstage_out, double *gamma_trace,
                           double *inc_trace, double *particles_out, double *lik_out, double *prior_out) {
    int r = check_ready(ctx);
    if (r) return r;
    if (n < 0 || (n > 0 && (!theta || !streams || !neglog_out || !status_out)))
        return ctx->fail(SMCGPU_ERR_ARG, "fault_likelihood: bad arguments");
    if (n == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    if (ctx->cfg.patch_km > 0.0) {
        if (particles_out)
            return ctx->fail(SMCGPU_ERR_ARG, "the slip population needs a fixed mesh (patch_km = 0)");
        return uneven_eval(ctx, n, theta, seed, (const unsigned long long *)streams, neglog_out, status_out,
                           nstage_out, gamma_trace, inc_trace);
    }
    const int nd = ctx->mesh.ndim_fault, ms = ctx->cfg.max_stages + 2;
    cudaStream_t s = ctx->stream;
    CU(ctx->d_theta.upload(theta, (size_t)n * nd, s), "upload theta");
    CU(ctx->d_streams.upload((const unsigned long long *)streams, n, s), "upload streams");
    CU(ctx->d_neglog.ensure(n), "alloc");
    CU(ctx->d_status.ensure(n), "alloc");
    NestedOpts opt;
    if (nstage_out || gamma_trace || inc_trace) {
        CU(ctx->d_nstage.ensure(n), "alloc");
        CU(ctx->d_trace.ensure((size_t)2 * n * ms), "alloc");
        CU(cudaMemsetAsync(ctx->d_trace.p, 0, (size_t)2 * n * ms * sizeof(double), s), "memset");
        opt.nstage = ctx->d_nstage.p;
        opt.trace_gamma = ctx->d_trace.p;
        opt.trace_inc = ctx->d_trace.p + (size_t)n * ms;
    }
    opt.particles_out = particles_out;
    opt.lik_out = lik_out;
    opt.prior_out = prior_out;
    r = nested_batch(ctx, n, ctx->d_theta.p, seed, ctx->d_streams.p, ctx->d_neglog.p, ctx->d_status.p, opt);
    if (r) return r;
    CU(cudaMemcpyAsync(neglog_out, ctx->d_neglog.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
    CU(cudaMemcpyAsync(status_out, ctx->d_status.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
    if (nstage_out)
        CU(cudaMemcpyAsync(nstage_out, ctx->d_nstage.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
    if (gamma_trace)
        CU(cudaMemcpyAsync(gamma_trace, ctx->d_trace.p, (size_t)n * ms * sizeof(double), cudaMemcpyDeviceToHost, s),
           "copy");
    if (inc_trace)
        CU(cudaMemcpyAsync(inc_trace, ctx->d_trace.p + (size_t)n * ms, (size_t)n * ms * sizeof(double),
                           cudaMemcpyDeviceToHost, s), "copy");
    CU(cudaStreamSynchronize(s), "sync");
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_fault_likelihood_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed,
                                                 const uint64_t *streams, double *neglog_out, int32_t *status_out) {
    if (!ctx) return SMCGPU_ERR_ARG;
    return likelihood_host(ctx, n_theta, theta, seed, streams, neglog_out, status_out, nullptr, nullptr, nullptr,
                           nullptr, nullptr, nullptr);
}

extern "C" int32_t smcgpu_fault_likelihood_trace(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed,
                                                 const uint64_t *streams, double *neglog_out, int32_t *status_out,
                                                 int32_t *nstage_out, double *gamma_trace, double *inc_trace) {
    if (!ctx) return SMCGPU_ERR_ARG;
    return likelihood_host(ctx, n_theta, theta, seed, streams, neglog_out, status_out, nstage_out, gamma_trace,
                           inc_trace, nullptr, nullptr, nullptr);
}

extern "C" int32_t smcgpu_fault_likelihood_posterior(smcgpu_ctx *ctx, const double *theta, uint64_t seed,
                                                     uint64_t stream, double *neglog_out, int32_t *status_out,
                                                     double *particles_out, double *likelihood_out,
                                                     double *prior_out) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!particles_out || !likelihood_out || !prior_out) return ctx->fail(SMCGPU_ERR_ARG, "posterior: null output");
    return likelihood_host(ctx, 1, theta, seed, &stream, neglog_out, status_out, nullptr, nullptr, nullptr,
                           particles_out, likelihood_out, prior_out);
}

// ---------------------------------------------------------------------------
// Outer SMC (fault_smc_exec, smc_fault.f90:785-1075), uniform prior box,
// driven from the host; every batch of nested evaluations is one device
// pipeline (Green's build, Gram, Gibbs init, inner SMC) over all thetas.
// ---------------------------------------------------------------------------
static int chol_lower_inplace(std::vector<double> &a, int n) {
    for (int j = 0; j < n; ++j) {
        double d = a[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= a[(size_t)k * n + j] * a[(size_t)k * n + j];
        if (!(d > 0.0)) return j + 1;
        d = std::sqrt(d);
        a[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double v = a[(size_t)j * n + i];
            for (int k = 0; k < j; ++k) v -= a[(size_t)k * n + i] * a[(size_t)k * n + j];
            a[(size_t)j * n + i] = v / d;
        }
    }
    return 0;
}

static double host_normal(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, uint64_t i, uint64_t d) {
    const double pi = 2.0 * std::asin(1.0);
    double r = smc::rng_uniform(seed, stream, purpose, stage, i, 2 * d);
    double sv = smc::rng_uniform(seed, stream, purpose, stage, i, 2 * d + 1);
    return std::sqrt(-2.0 * std::log(r)) * std::sin(2.0 * pi * sv);
}

static void write_stage_csv(const char *dir, int iter, const std::vector<double> &parts, const std::vector<double> &L,
                            int N, int nd) {
    // smc_fault.f90:923-936 / 1054-1067: file trim(output_dir)//iter//".csv",
    // one record per particle: ndim values and the likelihood, each f20.5
    std::string path = std::string(dir) + std::to_string(iter) + ".csv";
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return;
    std::string line;
    for (int i = 0; i < N; ++i) {
        line.clear();
        for (int d = 0; d < nd; ++d) line += smc::fortran_f(parts[(size_t)i * nd + d], 20, 5);
        line += smc::fortran_f(L[i], 20, 5);
        line += '\n';
        std::fputs(line.c_str(), f);
    }
    std::fclose(f);
}

// GSMC reference distribution q = N(qmean, qcov) (smc_fault.f90:9-52)
struct GsmcQ {
    const double *qmean, *qcov_chol, *qcov_inv;
    double log_qcov_det;
};

// dtrmv('l','n','n'): z := L z, L lower-triangular column-major (reference BLAS column order)
static void trmv_lower(const double *L, int nd, double *z) {
    for (int jj = nd - 1; jj >= 0; --jj) {
        double t = z[jj];
        for (int ii = nd - 1; ii > jj; --ii) z[ii] += t * L[(size_t)jj * nd + ii];
        z[jj] *= L[(size_t)jj * nd + jj];
    }
}

// fault_calc_neglog_q (smc_fault.f90:9-27), same loop order
static double neglog_q(const GsmcQ &q, const double *x, int nd) {
    const double pi = 2.0 * std::asin(1.0);
    std::vector<double> delta(nd);
    for (int d = 0; d < nd; ++d) delta[d] = x[d] - q.qmean[d];
    double tmp = 0.0;
    for (int j = 0; j < nd; ++j)
        for (int i = 0; i < nd; ++i) tmp = tmp + delta[i] * q.qcov_inv[(size_t)j * nd + i] * delta[j];
    return tmp / 2.0 + std::log(2.0 * pi) * nd / 2.0 + q.log_qcov_det / 2.0;
}

// Outer-SMC state after a completed stage: everything the next stage reads.
// Written as output_dir<iter>.state next to the stage CSV (full precision,
// where the CSV carries f20.5), so that a run can continue from any stage.
struct OuterState {
    int32_t nd = 0, N = 0, iter = 0, gsmc = 0, status = 0;
    double gamma = 0.0, evidence = 0.0;
    std::vector<double> parts, Ls, qs;
};
static const char STATE_MAGIC[8] = {'S', 'M', 'C', 'G', 'P', 'U', 'S', '1'};

static bool write_state(const char *dir, const OuterState &st) {
    const std::string path = std::string(dir) + std::to_string(st.iter) + ".state";
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    bool ok = std::fwrite(STATE_MAGIC, 1, 8, f) == 8;
    const int32_t hdr[5] = {st.nd, st.N, st.iter, st.gsmc, st.status};
    const double sc[2] = {st.gamma, st.evidence};
    ok = ok && std::fwrite(hdr, sizeof(int32_t), 5, f) == 5 && std::fwrite(sc, sizeof(double), 2, f) == 2;
    ok = ok && std::fwrite(st.parts.data(), sizeof(double), st.parts.size(), f) == st.parts.size();
    ok = ok && std::fwrite(st.Ls.data(), sizeof(double), st.Ls.size(), f) == st.Ls.size();
    ok = ok && std::fwrite(st.qs.data(), sizeof(double), st.qs.size(), f) == st.qs.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok && std::rename(tmp.c_str(), path.c_str()) == 0;
}

static std::string read_state(const char *path, OuterState &st) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return std::string("cannot open ") + path;
    char magic[8];
    int32_t hdr[5];
    double sc[2];
    std::string err;
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, STATE_MAGIC, 8) != 0) err = "not an outer-SMC state file";
    if (err.empty() && (std::fread(hdr, sizeof(int32_t), 5, f) != 5 || std::fread(sc, sizeof(double), 2, f) != 2))
        err = "truncated header";
    if (err.empty() && (hdr[0] < 1 || hdr[1] < 2 || hdr[2] < 0)) err = "bad header";
    if (err.empty()) {
        st.nd = hdr[0]; st.N = hdr[1]; st.iter = hdr[2]; st.gsmc = hdr[3]; st.status = hdr[4];
        st.gamma = sc[0]; st.evidence = sc[1];
        st.parts.resize((size_t)st.N * st.nd);
        st.Ls.resize(st.N);
        st.qs.resize(st.N);
        if (std::fread(st.parts.data(), sizeof(double), st.parts.size(), f) != st.parts.size() ||
            std::fread(st.Ls.data(), sizeof(double), st.Ls.size(), f) != st.Ls.size() ||
            std::fread(st.qs.data(), sizeof(double), st.qs.size(), f) != st.qs.size())
            err = "truncated state";
    }
    std::fclose(f);
    return err;
}

static int32_t outer_smc(smcgpu_ctx *ctx, const double *range, int32_t N, uint64_t seed, const char *output_dir,
                         const GsmcQ *gq, double *particles_out, double *likelihood_out, double *evidence_out,
                         int32_t *nstage_out, const OuterState *resume = nullptr) {
    if (!ctx) return SMCGPU_ERR_ARG;
    int r = check_ready(ctx);
    if (r) return r;
    if (!range || N < 2 || !evidence_out) return ctx->fail(SMCGPU_ERR_ARG, "fault_smc_exec: bad arguments");
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    if (output_dir) smc::mkdir_p(output_dir);
    const int nd = ctx->mesh.ndim_fault;
    const uint64_t OS = smc::OUTER_STREAM;
    cudaStream_t s = ctx->stream;
    std::vector<double> parts((size_t)N * nd), Ls(N), w(N), mean(nd), cov((size_t)nd * nd), qs(N, 0.0);
    std::vector<int32_t> assigned(N), sorted(N);
    int status = 0;
    smc::DevBuf<double> d_th, d_nl;
    smc::DevBuf<int> d_st, d_ns;
    smc::DevBuf<unsigned long long> d_sid;
    std::vector<int32_t> stv, nsv;
    // Inner stage count of each particle's latest evaluation: the cost key
    // that orders a batch (not part of the snapshot; a resumed run starts
    // unordered, which changes no result)
    std::vector<int> Ns(N, 0);
    // per-stage wall time and evaluations (smcgpu_outer_stage_times)
    ctx->outer_stage_s.clear();
    ctx->outer_stage_evals.clear();
    long long stage_evals = 0;
    auto stage_t0 = std::chrono::steady_clock::now();
    auto stage_done = [&]() {
        const auto t1 = std::chrono::steady_clock::now();
        ctx->outer_stage_s.push_back(std::chrono::duration<double>(t1 - stage_t0).count());
        ctx->outer_stage_evals.push_back(stage_evals);
        stage_evals = 0;
        stage_t0 = t1;
    };
    // nested evaluations of a batch; the status bits of every evaluation are
    // merged unless `used` marks the ones whose values are kept.  With `key`,
    // the batch runs in descending key order (the inner kernel's persistent
    // groups then take the costliest geometries first); results come back in
    // the caller's order, and the evaluations do not depend on the order.
    auto evaluate = [&](const std::vector<double> &th, const std::vector<unsigned long long> &sid,
                        std::vector<double> &out, const std::vector<char> *used = nullptr,
                        const std::vector<int> *key = nullptr, std::vector<int> *ns_out = nullptr) -> int {
        int nb = (int)sid.size();
        out.assign(nb, 0.0);
        if (ns_out) ns_out->assign(nb, 0);
        if (nb == 0) return SMCGPU_OK;
        stage_evals += nb;
        std::vector<int> perm(nb);
        for (int q = 0; q < nb; ++q) perm[q] = q;
        if (key) std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return (*key)[x] > (*key)[y]; });
        std::vector<double> th2((size_t)nb * nd);
        std::vector<unsigned long long> sid2(nb);
        for (int q = 0; q < nb; ++q) {
            std::memcpy(&th2[(size_t)q * nd], &th[(size_t)perm[q] * nd], nd * sizeof(double));
            sid2[q] = sid[perm[q]];
        }
        std::vector<double> out2(nb);
        std::vector<int32_t> st2(nb), ns2(nb);
        if (ctx->cfg.patch_km > 0.0) {
            int rr = uneven_eval(ctx, nb, th2.data(), seed, sid2.data(), out2.data(), st2.data(), ns2.data(), nullptr,
                                 nullptr);
            if (rr) return rr;
        } else {
        CU(d_th.upload(th2.data(), th2.size(), s), "upload");
        CU(d_sid.upload(sid2.data(), sid2.size(), s), "upload");
        CU(d_nl.ensure(nb), "alloc");
        CU(d_st.ensure(nb), "alloc");
        CU(d_ns.ensure(nb), "alloc");
        NestedOpts opt;
        opt.nstage = d_ns.p;
        int rr = nested_batch(ctx, nb, d_th.p, seed, d_sid.p, d_nl.p, d_st.p, opt);
        if (rr) return rr;
        CU(cudaMemcpyAsync(out2.data(), d_nl.p, nb * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
        CU(cudaMemcpyAsync(st2.data(), d_st.p, nb * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        CU(cudaMemcpyAsync(ns2.data(), d_ns.p, nb * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        CU(cudaStreamSynchronize(s), "sync");
        }
        stv.assign(nb, 0);
        for (int q = 0; q < nb; ++q) {
            out[perm[q]] = out2[q];
            stv[perm[q]] = st2[q];
            if (ns_out) (*ns_out)[perm[q]] = ns2[q];
        }
        for (int q = 0; q < nb; ++q)
            if (!used || (*used)[q]) status |= stv[q];
        return SMCGPU_OK;
    };
    double gamma = 0.0, evidence = 0.0;
    int iter = 1;
    auto save_state = [&](int it) {
        if (!output_dir) return;
        OuterState o;
        o.nd = nd; o.N = N; o.iter = it; o.gsmc = gq ? 1 : 0; o.status = status;
        o.gamma = gamma; o.evidence = evidence;
        o.parts = parts; o.Ls = Ls; o.qs = qs;
        if (!write_state(output_dir, o)) status |= SMCGPU_ST_SNAPSHOT_IO;
    };
    if (resume) {
        parts = resume->parts;
        Ls = resume->Ls;
        qs = resume->qs;
        gamma = resume->gamma;
        evidence = resume->evidence;
        iter = resume->iter + 1;
        status = resume->status;
    } else {
    // fault_sample_init_particles (smc_fault.f90:29-64): the prior box, or
    // N(qmean, qcov) in GSMC mode
    if (gq) {
        std::vector<double> z(nd);
        for (int i = 0; i < N; ++i) {
            for (int d = 0; d < nd; ++d) z[d] = host_normal(seed, OS, smc::RNG_OUT_QINIT, 0, i, d);
            trmv_lower(gq->qcov_chol, nd, z.data());
            for (int d = 0; d < nd; ++d) parts[(size_t)i * nd + d] = z[d] + gq->qmean[d];
        }
    } else {
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < nd; ++d) {
                double u = smc::rng_uniform(seed, OS, smc::RNG_OUT_INIT, 0, i, d);
                parts[(size_t)i * nd + d] = range[2 * d] + u * (range[2 * d + 1] - range[2 * d]);
            }
    }
    {
        std::vector<unsigned long long> sid(N);
        for (int i = 0; i < N; ++i) sid[i] = smc::eval_stream(0, 0, i);
        r = evaluate(parts, sid, Ls, nullptr, nullptr, &Ns);
        if (r) return r;
        // work_eval_init_particles (smc_fault.f90:350-353)
        if (gq)
            for (int i = 0; i < N; ++i) qs[i] = neglog_q(*gq, &parts[(size_t)i * nd], nd);
    }
    if (output_dir) write_stage_csv(output_dir, 0, parts, Ls, N, nd);
    save_state(0);
    stage_done();
    }
    CU(ctx->d_w.ensure(N), "alloc");
    CU(ctx->d_counts.ensure(N), "alloc");
    CU(ctx->d_flag.ensure(1), "alloc");
    while (1.0 - gamma > std::pow(10.0, -8.0)) {
        if (ctx->cfg.max_outer_stages != 0 && iter > std::max(ctx->cfg.max_outer_stages, 0)) break;
        Range stage_range("outer stage " + std::to_string(iter));
        // fault_find_next_gamma (smc_fault.f90:392-485); GSMC tempers L - q
        std::vector<double> nlr(N);
        for (int i = 0; i < N; ++i) nlr[i] = gq ? Ls[i] - qs[i] : Ls[i];
        double gprev = gamma, minL = nlr[0];
        for (int i = 0; i < N; ++i) minL = std::min(minL, nlr[i]);
        double lower = gprev, upper = 1.0, err = 1.0, dg;
        int cnt = 0;
        while (err > std::pow(10.0, -8.0)) {
            gamma = (lower + upper) / 2.0;
            dg = gamma - gprev;
            for (int i = 0; i < N; ++i) w[i] = std::exp(-dg * (nlr[i] - minL));
            double m = 0.0;
            for (int i = 0; i < N; ++i) m = m + w[i];
            m = m / N;
            double sd = 0.0;
            for (int i = 0; i < N; ++i) sd = sd + (w[i] - m) * (w[i] - m);
            sd = std::sqrt(sd / N);
            double cv = sd / m;
            if (cv > ctx->cfg.cv_outer) upper = gamma; else lower = gamma;
            err = std::fabs(cv - ctx->cfg.cv_outer);
            if (std::fabs(gamma - 1.0) < std::pow(10.0, -8.0)) break;
            if (cnt > 1000) break;
            cnt = cnt + 1;
        }
        double ev = 0.0;
        dg = gamma - gprev;
        for (int i = 0; i < N; ++i) ev = ev + std::exp(-dg * (nlr[i] - minL));
        ev = ev / N;
        evidence = evidence - std::log(ev) + dg * minL;
        // fault_normalize_weights, fault_calc_mean_particles, fault_calc_cov_particles
        double sum = 0.0;
        for (int i = 0; i < N; ++i) sum = sum + w[i];
        for (int i = 0; i < N; ++i) w[i] = w[i] / sum;
        for (int d = 0; d < nd; ++d) mean[d] = 0.0;
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < nd; ++d) mean[d] = mean[d] + w[i] * parts[(size_t)i * nd + d];
        std::fill(cov.begin(), cov.end(), 0.0);
        for (int i = 0; i < N; ++i) {
            double wt = w[i];
            for (int jd = 0; jd < nd; ++jd)
                for (int id = jd; id < nd; ++id)
                    cov[(size_t)jd * nd + id] = cov[(size_t)jd * nd + id] +
                        wt * (parts[(size_t)i * nd + id] - mean[id]) * (parts[(size_t)i * nd + jd] - mean[jd]);
        }
        for (double &c : cov) c = c * 0.04;
        if (chol_lower_inplace(cov, nd) != 0) status |= SMCGPU_ST_NONFINITE;
        // fault_resample_particles on the device (bit-exact binary128 counts)
        {
            double uh, ul;
            smc::rng_quad_uniform(seed, OS, smc::RNG_OUT_RES, iter, uh, ul);
            CU(ctx->d_w.upload(w.data(), N, s), "upload");
            CU(smc::launch_resample_counts(ctx->d_w.p, N, uh, ul, ctx->d_counts.p, ctx->d_flag.p, s), "resample");
            CU(cudaMemcpyAsync(assigned.data(), ctx->d_counts.p, N * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
            CU(cudaStreamSynchronize(s), "sync");
        }
        // fault_reorder_to_send with qsort_ (one rank: the sorted order itself)
        {
            std::vector<int32_t> ta = assigned;
            std::vector<double> tp = parts, tl = Ls, tq = qs;
            std::vector<int> tn = Ns;
            for (int i = 0; i < N; ++i) sorted[i] = i + 1;
            int32_t nn = N;
            smcgpu_qsort_(assigned.data(), sorted.data(), &nn);
            for (int k = 0; k < N; ++k) {
                int org = sorted[k] - 1;
                assigned[k] = ta[org];
                for (int d = 0; d < nd; ++d) parts[(size_t)k * nd + d] = tp[(size_t)org * nd + d];
                Ls[k] = tl[org];
                qs[k] = tq[org];
                Ns[k] = tn[org];
            }
        }
        // work_mcmc_sampling (smc_fault.f90:639-783): parents re-evaluated,
        // then chained random-walk proposals, batched by chain position.
        // Step j + 1 of a chain starts from the outcome of step j, so the
        // steps of a chain are sequential; late positions hold few chains and
        // leave the GPU idle.  A batch therefore covers the K positions rr ..
        // rr + K - 1 at once as each chain's decision tree: the proposal of a
        // later step is formed for both outcomes of every earlier step in the
        // window (2^m - 1 candidates for m steps), all are evaluated, and the
        // Metropolis decisions then walk down the tree.  Proposals and
        // evaluations are keyed by chain position, so the decisions, the
        // kept values and every output equal the step-by-step run; the
        // candidates off the taken path are discarded.
        std::vector<int32_t> start(N);
        start[0] = 0;
        for (int i = 0; i < N - 1; ++i) start[i + 1] = start[i] + assigned[i];
        std::vector<double> curp = parts, Lcur(N), newp((size_t)N * nd), newL(N), qcur = qs, newq(N, 0.0);
        std::vector<int> curN = Ns, newN(N, 0);
        int maxa = 0;
        for (int i = 0; i < N; ++i) maxa = std::max(maxa, (int)assigned[i]);
        int nparents = 0;
        for (int i = 0; i < N; ++i) nparents += assigned[i] > 0;
        // batch size of a window of K positions from rr: 2^min(K, remaining) - 1 per chain
        auto window_size = [&](int rr, int K) {
            long long n = rr == 0 ? nparents : 0;
            for (int i = 0; i < N; ++i) {
                const int m = std::min(K, (int)assigned[i] - rr);
                if (m > 0) n += (1LL << m) - 1;
            }
            return n;
        };
        // widen the window while the batch stays within one wave of the inner
        // kernel (two geometries per SM) or within the unwidened batch, or
        // while the added candidates are at most one wave: they cost at most
        // one more geometry time in a batch that already spans several waves,
        // and save a later batch, which costs at least its slowest geometry
        const long long wave = 2LL * std::max(ctx->nsm, 1);
        auto proposal = [&](const double *from, int j, double *x) {
            std::vector<double> z(nd);
            for (int d = 0; d < nd; ++d) z[d] = host_normal(seed, OS, smc::RNG_OUT_PROP, iter, j, d);
            trmv_lower(cov.data(), nd, z.data());
            for (int d = 0; d < nd; ++d) x[d] = from[d] + z[d];
            for (int d = 0; d < nd; ++d) {
                double lo = range[2 * d], hi = range[2 * d + 1];
                if (hi - lo > 1e-3) {
                    if (x[d] < lo) x[d] = std::min(2.0 * lo - x[d], hi);
                    if (x[d] > hi) x[d] = std::max(2.0 * hi - x[d], lo);
                }
            }
        };
        for (int rr = 0; rr < std::max(maxa, 1);) {
            int K = 1;
            const long long n1 = window_size(rr, 1);
            while (K < 8 && rr + K < maxa) {
                const long long nk = window_size(rr, K), nk1 = window_size(rr, K + 1);
                if (nk1 > std::max(wave, n1) && nk1 - nk > wave) break;
                ++K;
            }
            std::vector<double> cand;
            std::vector<unsigned long long> sid;
            std::vector<int> pidx;
            if (rr == 0) {
                // the parents' re-evaluation (smc_fault.f90:695-707) does not
                // depend on any Metropolis decision, so it shares the first
                // batch: parents first, then the proposals.  Parents without
                // children are skipped: their value is never used (the
                // reference computes and discards it).
                for (int i = 0; i < N; ++i) {
                    if (assigned[i] == 0) continue;
                    pidx.push_back(i);
                    cand.insert(cand.end(), parts.begin() + (size_t)i * nd, parts.begin() + (size_t)(i + 1) * nd);
                    sid.push_back(smc::eval_stream(iter, 0, i));
                }
            }
            const size_t npar = sid.size();
            std::vector<int> ckey;
            for (size_t q = 0; q < npar; ++q) ckey.push_back(Ns[pidx[q]]);
            // per chain: its first candidate index and its window depth; node
            // (l, b) of the tree is candidate first + 2^l - 1 + b, where bit t
            // of b is the outcome (1: accepted) of step rr + t
            std::vector<int> who, first, depth;
            for (int i = 0; i < N; ++i) {
                const int m = std::min(K, (int)assigned[i] - rr);
                if (m <= 0) continue;
                who.push_back(i);
                first.push_back((int)(sid.size() - npar));
                depth.push_back(m);
                const size_t base = sid.size();
                cand.resize(cand.size() + (((size_t)1 << m) - 1) * nd);
                sid.resize(sid.size() + ((size_t)1 << m) - 1);
                ckey.resize(sid.size(), curN[i]);
                for (int l = 0; l < m; ++l) {
                    const int j = start[i] + rr + l;
                    for (int b = 0; b < (1 << l); ++b) {
                        // the chain state before step rr + l on path b: the candidate
                        // of the last accepted step on the path, else the current state
                        const double *from = &curp[(size_t)i * nd];
                        for (int t = l - 1; t >= 0; --t)
                            if ((b >> t) & 1) {
                                from = &cand[(base + ((size_t)1 << t) - 1 + (b & ((1 << t) - 1))) * nd];
                                break;
                            }
                        const size_t node = base + ((size_t)1 << l) - 1 + b;
                        proposal(from, j, &cand[node * nd]);
                        sid[node] = smc::eval_stream(iter, 1, j);
                    }
                }
            }
            std::vector<double> Lall;
            std::vector<char> used(sid.size(), 0);   // filled below; statuses merged after the walk
            std::vector<int> nsall;
            r = evaluate(cand, sid, Lall, &used, &ckey, &nsall);
            if (r) return r;
            for (size_t q = 0; q < npar; ++q) {
                Lcur[pidx[q]] = Lall[q];
                curN[pidx[q]] = nsall[q];
                used[q] = 1;
            }
            for (size_t w2 = 0; w2 < who.size(); ++w2) {
                const int i = who[w2];
                int b = 0;
                for (int l = 0; l < depth[w2]; ++l) {
                    const int j = start[i] + rr + l;
                    const size_t node = npar + (size_t)first[w2] + ((size_t)1 << l) - 1 + b;
                    used[node] = 1;
                    const double *c = &cand[node * nd];
                    const double Lq = Lall[node];
                    double mh = smc::rng_uniform(seed, OS, smc::RNG_OUT_MH, iter, j, 0);
                    // work_mcmc_sampling's test (smc_fault.f90:748-771)
                    const double qc = gq ? neglog_q(*gq, c, nd) : 0.0;
                    const double lhs = gq ? gamma * (Lcur[i] - Lq) + (1.0 - gamma) * (qcur[i] - qc) : gamma * (Lcur[i] - Lq);
                    if (lhs > std::log(mh)) {
                        for (int d = 0; d < nd; ++d) curp[(size_t)i * nd + d] = c[d];
                        Lcur[i] = Lq;
                        qcur[i] = qc;
                        curN[i] = nsall[node];
                        b |= 1 << l;
                    }
                    newL[j] = Lcur[i];
                    newq[j] = qcur[i];
                    newN[j] = curN[i];
                    for (int d = 0; d < nd; ++d) newp[(size_t)j * nd + d] = curp[(size_t)i * nd + d];
                }
            }
            for (size_t q = 0; q < used.size(); ++q)
                if (used[q]) status |= stv[q];
            rr += K;
        }
        parts = newp;
        Ls = newL;
        qs = newq;
        Ns = newN;
        if (output_dir) write_stage_csv(output_dir, iter, parts, Ls, N, nd);
        save_state(iter);
        stage_done();
        iter = iter + 1;
        if (iter > 100000) break;
    }
    if (particles_out) std::memcpy(particles_out, parts.data(), parts.size() * sizeof(double));
    if (likelihood_out) std::memcpy(likelihood_out, Ls.data(), N * sizeof(double));
    *evidence_out = evidence;
    if (nstage_out) *nstage_out = iter - 1;
    if (status) ctx->err = "fault_smc_exec: status bits " + std::to_string(status);
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_fault_smc_exec(smcgpu_ctx *ctx, const double *range, int32_t N, uint64_t seed,
                                         const char *output_dir, double *particles_out, double *likelihood_out,
                                         double *evidence_out, int32_t *nstage_out) {
    return outer_smc(ctx, range, N, seed, output_dir, nullptr, particles_out, likelihood_out, evidence_out,
                     nstage_out);
}

extern "C" int32_t smcgpu_fault_smc_resume(smcgpu_ctx *ctx, const double *range, int32_t N, uint64_t seed,
                                           const char *output_dir, const char *state_path, const double *qmean,
                                           const double *qcov_chol, const double *qcov_inv, double log_qcov_det,
                                           double *particles_out, double *likelihood_out, double *evidence_out,
                                           int32_t *nstage_out) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!state_path) return ctx->fail(SMCGPU_ERR_ARG, "fault_smc_resume: state_path missing");
    OuterState st;
    std::string e = read_state(state_path, st);
    if (!e.empty()) return ctx->fail(SMCGPU_ERR_ARG, "fault_smc_resume: " + e);
    if (st.nd != ctx->mesh.ndim_fault || st.N != N)
        return ctx->fail(SMCGPU_ERR_ARG, "fault_smc_resume: state has a different ndim_fault or nparticle");
    const bool has_q = qmean && qcov_chol && qcov_inv;
    if ((st.gsmc != 0) != has_q)
        return ctx->fail(SMCGPU_ERR_ARG, "fault_smc_resume: GSMC parameters must be given exactly for a GSMC state");
    GsmcQ q{qmean, qcov_chol, qcov_inv, log_qcov_det};
    return outer_smc(ctx, range, N, seed, output_dir, has_q ? &q : nullptr, particles_out, likelihood_out,
                     evidence_out, nstage_out, &st);
}

extern "C" int32_t smcgpu_fault_smc_exec_gsmc(smcgpu_ctx *ctx, const double *range, int32_t N, uint64_t seed,
                                              const char *output_dir, const double *qmean, const double *qcov_chol,
                                              const double *qcov_inv, double log_qcov_det, double *particles_out,
                                              double *likelihood_out, double *evidence_out, int32_t *nstage_out) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!qmean || !qcov_chol || !qcov_inv) return ctx->fail(SMCGPU_ERR_ARG, "fault_smc_exec_gsmc: q missing");
    GsmcQ q{qmean, qcov_chol, qcov_inv, log_qcov_det};
    return outer_smc(ctx, range, N, seed, output_dir, &q, particles_out, likelihood_out, evidence_out, nstage_out);
}

extern "C" int32_t smcgpu_slip_map(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed,
                                   const uint64_t *streams, double *mean_slip_out, double *neglog_out,
                                   int32_t *status_out) {
    if (!ctx) return SMCGPU_ERR_ARG;
    int r = check_ready(ctx);
    if (r) return r;
    if (n_theta < 0 || (n_theta > 0 && (!theta || !streams || !mean_slip_out || !neglog_out || !status_out)))
        return ctx->fail(SMCGPU_ERR_ARG, "slip_map: bad arguments");
    if (ctx->cfg.patch_km > 0.0) return ctx->fail(SMCGPU_ERR_ARG, "slip_map needs a fixed mesh (patch_km = 0)");
    if (n_theta == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    const int nd = ctx->mesh.ndim_fault, D = ctx->mesh.D;
    cudaStream_t s = ctx->stream;
    smc::DevBuf<double> d_th, d_nl, d_mean;
    smc::DevBuf<int> d_st;
    smc::DevBuf<unsigned long long> d_sid;
    CU(d_th.upload(theta, (size_t)n_theta * nd, s), "upload theta");
    CU(d_sid.upload((const unsigned long long *)streams, n_theta, s), "upload streams");
    CU(d_nl.ensure(n_theta), "alloc");
    CU(d_st.ensure(n_theta), "alloc");
    CU(d_mean.ensure((size_t)n_theta * D), "alloc");
    NestedOpts opt;
    opt.mean_dev = d_mean.p;
    r = nested_batch(ctx, n_theta, d_th.p, seed, d_sid.p, d_nl.p, d_st.p, opt);
    if (r) return r;
    CU(cudaMemcpyAsync(mean_slip_out, d_mean.p, (size_t)n_theta * D * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy");
    CU(cudaMemcpyAsync(neglog_out, d_nl.p, (size_t)n_theta * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
    CU(cudaMemcpyAsync(status_out, d_st.p, (size_t)n_theta * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
    CU(cudaStreamSynchronize(s), "sync");
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_point_cloud(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, const double *slip,
                                      int32_t nr, double *points_out) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (n_theta < 0 || nr < 1 || (n_theta > 0 && (!theta || !slip || !points_out)))
        return ctx->fail(SMCGPU_ERR_ARG, "point_cloud: bad arguments");
    if (n_theta == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    const smc::MeshPattern &pm = ctx->mesh;
    const int nd = pm.ndim_fault;
    const int stride = ctx->cfg.basis == SMCGPU_BASIS_NODAL ? 2 * pm.nnode : pm.D;
    cudaStream_t s = ctx->stream;
    smc::DevBuf<double> d_th, d_slip, d_pts;
    smc::DevBuf<smc::PlaneGeom> d_pl;
    const size_t npts = (size_t)n_theta * pm.npatch * nr * nr;
    CU(d_th.upload(theta, (size_t)n_theta * nd, s), "upload theta");
    CU(d_slip.upload(slip, (size_t)n_theta * stride, s), "upload slip");
    CU(d_pl.ensure((size_t)n_theta * pm.nplane), "alloc");
    CU(d_pts.ensure(npts * 6), "alloc points");
    CU(smc::launch_planes(ctx->md, n_theta, d_th.p, d_pl.p, s), "planes kernel");
    CU(smc::launch_point_cloud(ctx->md, n_theta, d_pl.p, d_slip.p, stride, nr, d_pts.p, s), "point cloud kernel");
    CU(cudaMemcpyAsync(points_out, d_pts.p, npts * 6 * sizeof(double), cudaMemcpyDeviceToHost, s), "copy points");
    CU(cudaStreamSynchronize(s), "sync");
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_stats_reset(smcgpu_ctx *ctx, int32_t enable) {
    if (!ctx) return SMCGPU_ERR_ARG;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    auto &st = ctx->stats;
    double scratch = 0.0;
    CU(cudaStreamSynchronize(ctx->stream), "sync");
    CU(stats_resolve(st.inner_ev, scratch), "stats");
    CU(stats_resolve(st.batch_ev, scratch), "stats");
    st.inner_ms = st.batch_ms = 0.0;
    st.evals = 0;
    st.on = enable != 0;
    if (st.on) {
        CU(st.d_counters.ensure(2), "alloc counters");
        CU(cudaMemsetAsync(st.d_counters.p, 0, 2 * sizeof(unsigned long long), ctx->stream), "memset");
        CU(cudaStreamSynchronize(ctx->stream), "sync");
    }
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_stats_get(smcgpu_ctx *ctx, smcgpu_stats *out) {
    if (!ctx || !out) return SMCGPU_ERR_ARG;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    auto &st = ctx->stats;
    CU(cudaStreamSynchronize(ctx->stream), "sync");
    CU(stats_resolve(st.inner_ev, st.inner_ms), "stats");
    CU(stats_resolve(st.batch_ev, st.batch_ms), "stats");
    unsigned long long c[2] = {0, 0};
    if (st.d_counters.p) CU(cudaMemcpy(c, st.d_counters.p, sizeof(c), cudaMemcpyDeviceToHost), "copy counters");
    out->nested_evals = st.evals;
    out->inner_stages = (int64_t)c[0];
    out->inner_trajectories = (int64_t)c[1];
    out->inner_kernel_ms = st.inner_ms;
    out->nested_ms = st.batch_ms;
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_outer_stage_times(smcgpu_ctx *ctx, int32_t max, double *seconds, int64_t *evals,
                                            int32_t *n_out) {
    if (!ctx || !n_out || max < 0) return SMCGPU_ERR_ARG;
    const int n = (int)ctx->outer_stage_s.size();
    for (int k = 0; k < std::min(n, (int)max); ++k) {
        if (seconds) seconds[k] = ctx->outer_stage_s[k];
        if (evals) evals[k] = ctx->outer_stage_evals[k];
    }
    *n_out = n;
    return SMCGPU_OK;
}
