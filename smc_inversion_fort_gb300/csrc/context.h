// Context object behind the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/smcgpu.h"
#include "devbuf.h"
#include "kernels.h"
#include "mesh.h"

namespace smc {
// message of the last call that had no context (create, the file readers)
extern thread_local std::string g_create_err;
// Fortran "Fw.d" edit descriptor: right-aligned in w columns, w asterisks
// when the value does not fit, NaN / Infinity spelled as gfortran does
std::string fortran_f(double v, int w, int d);
// "mkdir -p" of a path (the reference shells out to it, main.f90:202-207)
void mkdir_p(const std::string &path);
}
struct smcgpu_ctx;
// per-geometry meshes: the child context of mesh nxi x neta (made on first
// use; it shares the parent's observations) and the release of all children
int smc_child_context(smcgpu_ctx *parent, int nxi, int neta, smcgpu_ctx **out);
void smc_drop_children(smcgpu_ctx *ctx);
// step engine and warps per geometry of a context's batches (SMCGPU_ENGINE_AUTO resolved)
void smc_resolve_engine(const smcgpu_ctx *ctx, int *engine, int *warps);

struct smcgpu_ctx {
    smcgpu_config cfg;
    smc::MeshPattern mesh;
    smc::MeshDev md{};
    cudaStream_t own_stream = nullptr, copy_stream = nullptr, stream = nullptr;
    std::string err;
    bool has_data = false;
    int nsm = 0;   // SMs of the device
    // host copy of the observation layout
    int nobs = 0, nsar = 0, ngnss = 0, npath = 0, nstation = 0;
    std::vector<int> nsar_index0;  // zero-based path starts, npath+1
    std::vector<double> sar_whiten;   // per path lower-triangular W with W^T W = Sigma^-1 (col-major)
    std::vector<long long> sar_off;
    std::vector<double> dvec_h;
    double dsd_sar = 0.0, dsd_gnss = 0.0;  // whitened data norms (without sigma2 scalings)

    // pattern tables
    smc::DevBuf<int> d_dof_of_node, d_l_col, d_l_plane, d_lt_row, d_lt_plane, d_ll_ptr, d_ll_col;
    smc::DevBuf<int> d_gb_order, d_gb_lvl_ptr;
    smc::DevBuf<signed char> d_l_k, d_lt_k;
    // observations
    smc::DevBuf<double> d_st_x, d_st_y, d_obs_e, d_obs_sigma, d_dvec, d_sar_w, d_dx, d_roww;
    smc::DevBuf<int> d_st_row, d_st_nrow, d_nsar_index;
    smc::DevBuf<long long> d_sar_off;

    // batch work buffers
    smc::DevBuf<double> d_theta;
    smc::DevBuf<smc::PlaneGeom> d_planes;
    smc::DevBuf<char> d_gchunk[2];
    smc::DevBuf<double> d_gmat, d_gw, d_A, d_b, d_dsd, d_lval, d_ltval, d_llval;
    smc::DevBuf<smc::ThetaAux> d_aux;
    smc::DevBuf<double> d_neglog;
    smc::DevBuf<int> d_status;
    smc::DevBuf<unsigned long long> d_streams;
    smc::DevBuf<double> d_parts, d_parts_new, d_dbuf, d_trace;
    smc::DevBuf<float> d_A32, d_lv32, d_ll32;
    smc::DevBuf<int> d_queue;     // geometry queue of the persistent inner kernel
    smc::DevBuf<uint4> d_afrag;   // stage matrices in MMA-fragment order (MIXED, 128 < D <= 256)
    smc::DevBuf<char> d_mgl, d_glxc;   // global-matrix engine: stage matrices, slot chain states
    smc::DevBuf<int> d_ibuf, d_nstage_tmp, d_nstage;
    smc::DevBuf<double> d_w;
    smc::DevBuf<int> d_counts, d_flag;
    cudaEvent_t ev_done[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};

    // run statistics (smcgpu_stats_*): off unless enabled; device event pairs
    // around the inner kernel and the whole nested batch, resolved lazily
    struct Stats {
        bool on = false;
        std::vector<cudaEvent_t> inner_ev, batch_ev;   // start, stop, start, stop, ...
        double inner_ms = 0.0, batch_ms = 0.0;
        long long evals = 0;
        smc::DevBuf<unsigned long long> d_counters;    // [0] stages, [1] trajectories
    } stats;
    // per-geometry meshes (cfg.patch_km > 0): one child context per mesh, made
    // on first use; a child borrows the parent's observation buffers
    smcgpu_ctx *parent = nullptr;
    std::map<long long, smcgpu_ctx *> children;
    // engine table of SMCGPU_ENGINE_AUTO, per precision (0 FP64, 1 MIXED)
    std::vector<int> eng_dmax[2], eng_engine[2], eng_warps[2];
    // per-stage wall seconds and nested evaluations of the last fault_smc_exec
    std::vector<double> outer_stage_s;
    std::vector<long long> outer_stage_evals;

    // the whitened-observation tables of the gram kernel (a child context
    // borrows its parent's)
    const double *obs_roww() const { return parent ? parent->d_roww.p : d_roww.p; }
    const double *obs_dx() const { return parent ? parent->d_dx.p : d_dx.p; }

    int fail(int code, const std::string &msg) {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *where) {
        err = std::string(where) + ": " + cudaGetErrorString(e);
        return SMCGPU_ERR_CUDA;
    }
};
