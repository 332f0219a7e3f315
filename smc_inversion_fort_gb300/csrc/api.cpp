// C ABI entry points (include/smcgpu.h): context, observation upload and the
// Green's-function batch.  The nested-likelihood and outer-SMC entry points
// live in driver.cpp.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "context.h"

using smc::DevBuf;

namespace smc {
thread_local std::string g_create_err;
}
using smc::g_create_err;

#define CU(call, where)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return ctx->cuda_fail(e_, where); \
    } while (0)

extern "C" int32_t smcgpu_default_config(smcgpu_config *cfg) {
    if (!cfg) return SMCGPU_ERR_ARG;
    memset(cfg, 0, sizeof(*cfg));
    cfg->layout = SMCGPU_LAYOUT_TRACE;
    cfg->basis = SMCGPU_BASIS_NODAL;
    cfg->nplane = 1;
    cfg->nxi[0] = 8;
    cfg->neta[0] = 4;
    cfg->xmin = -20.0;
    cfg->xmax = 20.0;
    cfg->zmin = -20.0;
    cfg->nquad = 2;
    cfg->alpha = 2.0 / 3.0;
    cfg->max_slip = 4.0;
    cfg->nparticle_slip = 500;
    cfg->ntau = 50;
    cfg->tuning_factor = 5;
    cfg->max_stages = 200;
    cfg->cv_inner = 2.0;
    cfg->cv_outer = 0.2;
    cfg->sar_corr_len = 10.0;
    cfg->precision = SMCGPU_PREC_FP64;
    cfg->device = 0;
    return SMCGPU_OK;
}

static void refresh_md(smcgpu_ctx *ctx) {
    smc::MeshDev &m = ctx->md;
    const smc::MeshPattern &p = ctx->mesh;
    m.layout = p.layout; m.basis = p.basis; m.nquad = p.nquad; m.rect_hyper = p.rect_hyper;
    m.ndim_fault = p.ndim_fault; m.nplane = p.nplane; m.nnode = p.nnode; m.npatch = p.npatch;
    m.ndof = p.ndof; m.D = p.D; m.npt = p.npt; m.nrow = p.nrow;
    for (int i = 0; i < smc::MAXP; ++i) {
        m.nxi[i] = p.nxi[i]; m.neta[i] = p.neta[i]; m.xbend[i] = ctx->cfg.xbend[i];
    }
    for (int i = 0; i <= smc::MAXP; ++i) { m.node_off[i] = p.node_off[i]; m.patch_off[i] = p.patch_off[i]; }
    m.xmin = ctx->cfg.xmin; m.xmax = ctx->cfg.xmax; m.zmin = ctx->cfg.zmin; m.alpha = ctx->cfg.alpha;
    for (int i = 0; i < smc::MAXQ; ++i) {
        m.gq_x[i] = i < (int)p.gq_x.size() ? p.gq_x[i] : 0.0;
        m.gq_w[i] = i < (int)p.gq_w.size() ? p.gq_w[i] : 0.0;
    }
    m.dof_of_node = ctx->d_dof_of_node.p;
    m.l_col = ctx->d_l_col.p; m.l_k = ctx->d_l_k.p; m.l_plane = ctx->d_l_plane.p;
    m.lt_row = ctx->d_lt_row.p; m.lt_k = ctx->d_lt_k.p; m.lt_plane = ctx->d_lt_plane.p;
    m.ll_ptr = ctx->d_ll_ptr.p; m.ll_col = ctx->d_ll_col.p;
    m.ll_nnz = (int)p.ll_col.size(); m.ll_maxrow = p.ll_maxrow;
    m.gb_order = ctx->d_gb_order.p; m.gb_lvl_ptr = ctx->d_gb_lvl_ptr.p;
    m.gb_nlevel = (int)p.gb_lvl_ptr.size() - 1;
    m.nobs = ctx->nobs; m.nsar = ctx->nsar; m.ngnss = ctx->ngnss; m.nstation = ctx->nstation; m.npath = ctx->npath;
    m.st_x = ctx->d_st_x.p; m.st_y = ctx->d_st_y.p; m.st_row = ctx->d_st_row.p; m.st_nrow = ctx->d_st_nrow.p;
    m.obs_e = ctx->d_obs_e.p; m.obs_sigma = ctx->d_obs_sigma.p; m.dvec = ctx->d_dvec.p;
    m.nsar_index = ctx->d_nsar_index.p; m.sar_inv = ctx->d_sar_w.p; m.sar_off = ctx->d_sar_off.p;
}

extern "C" int32_t smcgpu_gibbs_levels(const smcgpu_config *cfg, int32_t *D, int32_t *nlevel, int32_t *order,
                                       int32_t *level_ptr) {
    if (!cfg || !D || !nlevel || (order && !level_ptr)) return SMCGPU_ERR_ARG;
    smc::MeshPattern p;
    if (!p.build(*cfg).empty()) return SMCGPU_ERR_ARG;
    *D = p.D;
    *nlevel = (int32_t)p.gb_lvl_ptr.size() - 1;
    if (order) {
        std::copy(p.gb_order.begin(), p.gb_order.end(), order);
        std::copy(p.gb_lvl_ptr.begin(), p.gb_lvl_ptr.end(), level_ptr);
    }
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_create(const smcgpu_config *cfg, smcgpu_ctx **out) {
    g_create_err.clear();
    if (!cfg || !out) { g_create_err = "null argument"; return SMCGPU_ERR_ARG; }
    *out = nullptr;
    smcgpu_ctx *ctx = new smcgpu_ctx();
    ctx->cfg = *cfg;
    std::string e = ctx->mesh.build(*cfg);
    if (e.empty() && cfg->basis == SMCGPU_BASIS_NODAL)
        for (int ip = 0; ip < cfg->nplane; ++ip)
            if (cfg->nxi[ip] > 32) e = "nodal basis supports nxi <= 32 per plane";
    if (e.empty() && (cfg->nparticle_slip < 2 || cfg->ntau < 1 || cfg->tuning_factor < 1 || cfg->max_stages < 0))
        e = "invalid SMC settings";
    if (e.empty() && !(cfg->max_slip > 0.0)) e = "max_slip must be positive";
    if (e.empty() && cfg->inner_warps != 0 && cfg->inner_warps != 1 && cfg->inner_warps != 2 &&
        cfg->inner_warps != 4 && cfg->inner_warps != 8)
        e = "inner_warps must be 0, 1, 2, 4 or 8";
    if (e.empty() && (cfg->inner_engine < SMCGPU_ENGINE_MMA || cfg->inner_engine > SMCGPU_ENGINE_AUTO))
        e = "inner_engine must be SMCGPU_ENGINE_MMA, _CUDA, _TCGEN05, _GLOBAL or _AUTO";
    if (e.empty() && !(cfg->patch_km >= 0.0)) e = "patch_km must be >= 0";
    if (e.empty() && cfg->patch_km > 0.0 && cfg->layout != SMCGPU_LAYOUT_RECT)
        e = "per-geometry meshes (patch_km > 0) need the rectangle layout";
    if (!e.empty()) { g_create_err = e; delete ctx; return SMCGPU_ERR_ARG; }
    cudaError_t ce = cudaSetDevice(cfg->device);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, cfg->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && ce == cudaSuccess; ++i) {
        ce = cudaEventCreateWithFlags(&ctx->ev_done[i], cudaEventDisableTiming);
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&ctx->ev_copied[i], cudaEventDisableTiming);
    }
    if (ce != cudaSuccess) {
        g_create_err = std::string("cuda: ") + cudaGetErrorString(ce);
        smcgpu_destroy(ctx);
        return SMCGPU_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    const smc::MeshPattern &p = ctx->mesh;
    cudaStream_t s = ctx->stream;
    ce = cudaSuccess;
    auto up = [&](cudaError_t r) { if (ce == cudaSuccess) ce = r; };
    up(ctx->d_dof_of_node.upload(p.dof_of_node, s));
    up(ctx->d_l_col.upload(p.l_col, s));
    up(ctx->d_l_k.upload(p.l_k, s));
    up(ctx->d_l_plane.upload(p.l_plane, s));
    up(ctx->d_lt_row.upload(p.lt_row, s));
    up(ctx->d_lt_k.upload(p.lt_k, s));
    up(ctx->d_lt_plane.upload(p.lt_plane, s));
    up(ctx->d_ll_ptr.upload(p.ll_ptr, s));
    up(ctx->d_ll_col.upload(p.ll_col, s));
    up(ctx->d_gb_order.upload(p.gb_order, s));
    up(ctx->d_gb_lvl_ptr.upload(p.gb_lvl_ptr, s));
    up(cudaStreamSynchronize(s));
    if (ce != cudaSuccess) {
        g_create_err = std::string("cuda: ") + cudaGetErrorString(ce);
        smcgpu_destroy(ctx);
        return SMCGPU_ERR_CUDA;
    }
    refresh_md(ctx);
    *out = ctx;
    return SMCGPU_OK;
}

int smc_child_context(smcgpu_ctx *parent, int nxi, int neta, smcgpu_ctx **out) {
    const long long key = (long long)nxi * 4096 + neta;
    auto it = parent->children.find(key);
    if (it != parent->children.end()) {
        *out = it->second;
        return SMCGPU_OK;
    }
    smcgpu_config c = parent->cfg;
    c.nxi[0] = nxi;
    c.neta[0] = neta;
    c.patch_km = 0.0;
    smcgpu_ctx *ch = nullptr;
    int r = smcgpu_create(&c, &ch);
    if (r != SMCGPU_OK)
        return parent->fail(r, "mesh " + std::to_string(nxi) + "x" + std::to_string(neta) + ": " + g_create_err);
    ch->parent = parent;
    for (int k = 0; k < 2; ++k) {
        ch->eng_dmax[k] = parent->eng_dmax[k];
        ch->eng_engine[k] = parent->eng_engine[k];
        ch->eng_warps[k] = parent->eng_warps[k];
    }
    ch->nobs = parent->nobs; ch->nsar = parent->nsar; ch->ngnss = parent->ngnss; ch->npath = parent->npath;
    ch->nstation = parent->nstation;
    ch->nsar_index0 = parent->nsar_index0;
    ch->dsd_sar = parent->dsd_sar;
    ch->dsd_gnss = parent->dsd_gnss;
    ch->has_data = true;
    refresh_md(ch);
    const smc::MeshDev &pm = parent->md;
    smc::MeshDev &m = ch->md;
    m.st_x = pm.st_x; m.st_y = pm.st_y; m.st_row = pm.st_row; m.st_nrow = pm.st_nrow;
    m.obs_e = pm.obs_e; m.obs_sigma = pm.obs_sigma; m.dvec = pm.dvec;
    m.nsar_index = pm.nsar_index; m.sar_inv = pm.sar_inv; m.sar_off = pm.sar_off;
    parent->children[key] = ch;
    *out = ch;
    return SMCGPU_OK;
}

void smc_drop_children(smcgpu_ctx *ctx) {
    for (auto &kv : ctx->children) smcgpu_destroy(kv.second);
    ctx->children.clear();
}

extern "C" int32_t smcgpu_set_engine_table(smcgpu_ctx *ctx, int32_t precision, int32_t n, const int32_t *dmax,
                                           const int32_t *engine, const int32_t *warps) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (precision != SMCGPU_PREC_FP64 && precision != SMCGPU_PREC_MIXED)
        return ctx->fail(SMCGPU_ERR_ARG, "engine table: precision must be FP64 or MIXED");
    if (n < 0 || (n > 0 && (!dmax || !engine || !warps))) return ctx->fail(SMCGPU_ERR_ARG, "engine table: bad arguments");
    const int pi = precision == SMCGPU_PREC_MIXED ? 1 : 0;
    for (int k = 0; k < n; ++k) {
        if (k > 0 && dmax[k] <= dmax[k - 1]) return ctx->fail(SMCGPU_ERR_ARG, "engine table: dmax must ascend");
        if (engine[k] < SMCGPU_ENGINE_MMA || engine[k] > SMCGPU_ENGINE_GLOBAL)
            return ctx->fail(SMCGPU_ERR_ARG, "engine table: engine must be MMA, CUDA, TCGEN05 or GLOBAL");
        if (pi == 0 && engine[k] != SMCGPU_ENGINE_CUDA && engine[k] != SMCGPU_ENGINE_GLOBAL)
            return ctx->fail(SMCGPU_ERR_ARG, "engine table: FP64 runs on the CUDA-core or global-matrix engine");
        if (warps[k] != 0 && warps[k] != 1 && warps[k] != 2 && warps[k] != 4 && warps[k] != 8)
            return ctx->fail(SMCGPU_ERR_ARG, "engine table: warps must be 0, 1, 2, 4 or 8");
    }
    ctx->eng_dmax[pi].assign(dmax, dmax + n);
    ctx->eng_engine[pi].assign(engine, engine + n);
    ctx->eng_warps[pi].assign(warps, warps + n);
    for (auto &kv : ctx->children) {
        kv.second->eng_dmax[pi] = ctx->eng_dmax[pi];
        kv.second->eng_engine[pi] = ctx->eng_engine[pi];
        kv.second->eng_warps[pi] = ctx->eng_warps[pi];
    }
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_destroy(smcgpu_ctx *ctx) {
    if (!ctx) return SMCGPU_OK;
    smc_drop_children(ctx);
    cudaSetDevice(ctx->cfg.device);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (cudaEvent_t e : ctx->stats.inner_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->stats.batch_ev) cudaEventDestroy(e);
    for (int i = 0; i < 2; ++i) {
        if (ctx->ev_done[i]) cudaEventDestroy(ctx->ev_done[i]);
        if (ctx->ev_copied[i]) cudaEventDestroy(ctx->ev_copied[i]);
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    delete ctx;
    return SMCGPU_OK;
}

extern "C" const char *smcgpu_last_error(const smcgpu_ctx *ctx) {
    if (!ctx) return g_create_err.c_str();
    return ctx->err.c_str();
}

extern "C" int32_t smcgpu_set_stream(smcgpu_ctx *ctx, void *stream) {
    if (!ctx) return SMCGPU_ERR_ARG;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_dims(const smcgpu_ctx *ctx, int32_t *ndim_fault, int32_t *D, int32_t *nobs, int32_t *nrow_l) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (ndim_fault) *ndim_fault = ctx->mesh.ndim_fault;
    if (D) *D = ctx->mesh.D;
    if (nobs) *nobs = ctx->nobs;
    if (nrow_l) *nrow_l = ctx->mesh.nrow;
    return SMCGPU_OK;
}

// Lower Cholesky factor (column-major) in place; returns 0 or the failing column+1.
static int chol_lower(std::vector<double> &a, int n) {
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

extern "C" int32_t smcgpu_set_data(smcgpu_ctx *ctx, int32_t nobs, const double *obs_points, const double *obs_unitvec,
                                   const double *obs_sigma, const double *dvec, int32_t npath,
                                   const int32_t *nsar_index, int32_t ngnss) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (nobs <= 0 || !obs_points || !obs_unitvec || !obs_sigma || !dvec || npath < 0 || ngnss < 0)
        return ctx->fail(SMCGPU_ERR_ARG, "set_data: invalid arguments");
    smc_drop_children(ctx);   // they borrow the observation buffers about to be replaced
    if (npath > 0 && !nsar_index) return ctx->fail(SMCGPU_ERR_ARG, "set_data: nsar_index missing");
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    std::vector<int> idx0(npath + 1, 0);
    for (int p = 0; p <= npath; ++p) idx0[p] = nsar_index[p] - 1;  // reference's 1-based table
    if (npath > 0 && idx0[0] != 0) return ctx->fail(SMCGPU_ERR_ARG, "set_data: nsar_index(1) must be 1");
    for (int p = 0; p < npath; ++p)
        if (idx0[p + 1] < idx0[p]) return ctx->fail(SMCGPU_ERR_ARG, "set_data: nsar_index not monotone");
    int nsar = npath > 0 ? idx0[npath] : 0;
    if (nsar + 3 * ngnss != nobs) return ctx->fail(SMCGPU_ERR_ARG, "set_data: nobs != nsar_total + 3*ngnss");
    for (int i = 0; i < nobs; ++i) {
        if (!(obs_sigma[i] > 0.0) || !std::isfinite(obs_sigma[i]))
            return ctx->fail(SMCGPU_ERR_ARG, "set_data: obs_sigma must be positive and finite (row " +
                                                 std::to_string(i + 1) + ")");
        if (!std::isfinite(dvec[i]) || !std::isfinite(obs_points[2 * i]) || !std::isfinite(obs_points[2 * i + 1]) ||
            !std::isfinite(obs_unitvec[3 * i]) || !std::isfinite(obs_unitvec[3 * i + 1]) ||
            !std::isfinite(obs_unitvec[3 * i + 2]))
            return ctx->fail(SMCGPU_ERR_ARG, "set_data: non-finite observation (row " + std::to_string(i + 1) + ")");
    }
    ctx->nobs = nobs; ctx->nsar = nsar; ctx->ngnss = ngnss; ctx->npath = npath;
    ctx->nstation = nsar + ngnss;
    ctx->nsar_index0 = idx0;
    std::vector<double> sx(ctx->nstation), sy(ctx->nstation);
    std::vector<int> srow(ctx->nstation), snrow(ctx->nstation);
    for (int i = 0; i < nsar; ++i) { sx[i] = obs_points[2 * i]; sy[i] = obs_points[2 * i + 1]; srow[i] = i; snrow[i] = 1; }
    for (int k = 0; k < ngnss; ++k) {
        int r = nsar + 3 * k;
        sx[nsar + k] = obs_points[2 * r]; sy[nsar + k] = obs_points[2 * r + 1];
        srow[nsar + k] = r; snrow[nsar + k] = 3;
    }
    // Sigma_SAR per path (init.f90:93-111, including its one-row offset in
    // the obs_sigma index, clamped at the last row), whitened by its Cholesky
    // factor: W = C^-1 with Sigma = C C^T, so W^T W = Sigma^-1.
    ctx->sar_whiten.clear();
    ctx->sar_off.assign(std::max(npath, 1), 0);
    std::vector<double> dx(nobs, 0.0), roww(nobs, 0.0);
    ctx->dsd_sar = 0.0;
    for (int p = 0; p < npath; ++p) {
        int st = idx0[p], n = idx0[p + 1] - idx0[p];
        std::vector<double> a((size_t)n * n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double xi = obs_points[2 * (st + i)], yi = obs_points[2 * (st + i) + 1];
                double xj = obs_points[2 * (st + j)], yj = obs_points[2 * (st + j) + 1];
                double dist = std::sqrt((xi - xj) * (xi - xj) + (yi - yj) * (yi - yj));
                int ri = std::min(st + i + 1, nobs - 1), rj = std::min(st + j + 1, nobs - 1);
                a[(size_t)j * n + i] = obs_sigma[ri] * obs_sigma[rj] * std::exp(-dist / ctx->cfg.sar_corr_len);
            }
        if (chol_lower(a, n) != 0) return ctx->fail(SMCGPU_ERR_ARG, "set_data: SAR covariance not positive definite");
        // W = C^-1 (lower), column by column
        std::vector<double> w((size_t)n * n, 0.0);
        for (int c = 0; c < n; ++c) {
            for (int i = c; i < n; ++i) {
                double v = (i == c) ? 1.0 : 0.0;
                for (int k = c; k < i; ++k) v -= a[(size_t)k * n + i] * w[(size_t)c * n + k];
                w[(size_t)c * n + i] = v / a[(size_t)i * n + i];
            }
        }
        ctx->sar_off[p] = (long long)ctx->sar_whiten.size();
        ctx->sar_whiten.insert(ctx->sar_whiten.end(), w.begin(), w.end());
        for (int i = 0; i < n; ++i) {
            double v = 0.0;
            for (int k = 0; k <= i; ++k) v += w[(size_t)k * n + i] * dvec[st + k];
            dx[st + i] = v;
            roww[st + i] = 1.0;
            ctx->dsd_sar += v * v;
        }
    }
    ctx->dsd_gnss = 0.0;
    for (int r = nsar; r < nobs; ++r) {
        dx[r] = dvec[r];
        roww[r] = 1.0 / (obs_sigma[r] * obs_sigma[r]);
        ctx->dsd_gnss += dvec[r] * dvec[r] * roww[r];
    }
    ctx->dvec_h.assign(dvec, dvec + nobs);
    cudaStream_t s = ctx->stream;
    std::vector<double> e3(obs_unitvec, obs_unitvec + 3 * (size_t)nobs);
    std::vector<double> sg(obs_sigma, obs_sigma + nobs), dv(dvec, dvec + nobs);
    CU(ctx->d_st_x.upload(sx, s), "upload");
    CU(ctx->d_st_y.upload(sy, s), "upload");
    CU(ctx->d_st_row.upload(srow, s), "upload");
    CU(ctx->d_st_nrow.upload(snrow, s), "upload");
    CU(ctx->d_obs_e.upload(e3, s), "upload");
    CU(ctx->d_obs_sigma.upload(sg, s), "upload");
    CU(ctx->d_dvec.upload(dv, s), "upload");
    CU(ctx->d_dx.upload(dx, s), "upload");
    CU(ctx->d_roww.upload(roww, s), "upload");
    CU(ctx->d_nsar_index.upload(idx0, s), "upload");
    if (ctx->sar_whiten.empty()) ctx->sar_whiten.push_back(0.0);
    CU(ctx->d_sar_w.upload(ctx->sar_whiten, s), "upload");
    CU(ctx->d_sar_off.upload(ctx->sar_off, s), "upload");
    CU(cudaStreamSynchronize(s), "set_data sync");
    ctx->has_data = true;
    refresh_md(ctx);
    return SMCGPU_OK;
}

static size_t gelem_bytes(int precision) { return precision == SMCGPU_PREC_FP32 ? sizeof(float) : sizeof(double); }

extern "C" int32_t smcgpu_greens_batch_dev(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                           int32_t precision, void *gmat_dev) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!ctx->has_data) return ctx->fail(SMCGPU_ERR_NODATA, "greens: set_data not called");
    if (n_theta < 0 || (n_theta > 0 && (!theta_dev || !gmat_dev))) return ctx->fail(SMCGPU_ERR_ARG, "greens: bad arguments");
    if (precision != SMCGPU_PREC_FP64 && precision != SMCGPU_PREC_FP32)
        return ctx->fail(SMCGPU_ERR_ARG, "greens: precision must be FP64 or FP32");
    if (n_theta == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    CU(ctx->d_planes.ensure((size_t)n_theta * ctx->mesh.nplane), "alloc planes");
    CU(smc::launch_planes(ctx->md, n_theta, theta_dev, ctx->d_planes.p, ctx->stream), "planes kernel");
    CU(smc::launch_greens(ctx->md, n_theta, ctx->d_planes.p, precision, gmat_dev, ctx->stream), "greens kernel");
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_greens_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, int32_t precision,
                                       void *gmat) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!ctx->has_data) return ctx->fail(SMCGPU_ERR_NODATA, "greens: set_data not called");
    if (n_theta < 0 || (n_theta > 0 && (!theta || !gmat))) return ctx->fail(SMCGPU_ERR_ARG, "greens: bad arguments");
    if (precision != SMCGPU_PREC_FP64 && precision != SMCGPU_PREC_FP32)
        return ctx->fail(SMCGPU_ERR_ARG, "greens: precision must be FP64 or FP32");
    if (n_theta == 0) return SMCGPU_OK;
    CU(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    const int nd = ctx->mesh.ndim_fault;
    const size_t per = (size_t)ctx->mesh.D * ctx->nobs * gelem_bytes(precision);
    // chunks of at most ~1 GiB of output, double-buffered: the D2H copy of
    // chunk k overlaps the build of chunk k+1
    int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)n_theta, (size_t)(1u << 30) / std::max<size_t>(per, 1)));
    CU(ctx->d_theta.upload(theta, (size_t)n_theta * nd, ctx->stream), "upload theta");
    CU(ctx->d_planes.ensure((size_t)chunk * ctx->mesh.nplane), "alloc planes");
    for (int b = 0; b < 2; ++b) CU(ctx->d_gchunk[b].ensure((size_t)chunk * per), "alloc gmat chunk");
    int k = 0;
    for (int t0 = 0; t0 < n_theta; t0 += chunk, ++k) {
        int nb = std::min(chunk, n_theta - t0);
        int b = k & 1;
        if (k >= 2) CU(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[b], 0), "wait");
        CU(smc::launch_planes(ctx->md, nb, ctx->d_theta.p + (size_t)t0 * nd, ctx->d_planes.p, ctx->stream), "planes kernel");
        CU(smc::launch_greens(ctx->md, nb, ctx->d_planes.p, precision, ctx->d_gchunk[b].p, ctx->stream), "greens kernel");
        CU(cudaEventRecord(ctx->ev_done[b], ctx->stream), "record");
        CU(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_done[b], 0), "wait");
        CU(cudaMemcpyAsync((char *)gmat + (size_t)t0 * per, ctx->d_gchunk[b].p, (size_t)nb * per,
                           cudaMemcpyDeviceToHost, ctx->copy_stream), "copy gmat");
        CU(cudaEventRecord(ctx->ev_copied[b], ctx->copy_stream), "record");
    }
    CU(cudaStreamSynchronize(ctx->copy_stream), "sync");
    CU(cudaStreamSynchronize(ctx->stream), "sync");
    return SMCGPU_OK;
}

extern "C" void smcgpu_qsort_(int32_t *arr, int32_t *index, int32_t *n) {
    // sort.cpp:3-7: order the 1-based index[] by arr[index-1], descending,
    // with std::sort (introsort, not stable) and the same comparator
    if (!arr || !index || !n || *n <= 1) return;
    std::sort(index, index + (*n), [&](int32_t a, int32_t b) { return arr[a - 1] > arr[b - 1]; });
}
