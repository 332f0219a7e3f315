/*
 * smcgpu.h -- C ABI of the GB300 nested-SMC fault-geometry / slip inversion.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int32_t status (SMCGPU_OK = 0) and never exits, stops or traps.  Arrays are
 * in the reference's Fortran layouts (column-major, first index fastest), so a
 * Fortran caller passes its own arrays through ISO_C_BINDING unchanged (a
 * `bind(C)` interface per entry point, as for sort.cpp's qsort_).  Host pointers are
 * owned by the caller and not retained past a call.  One context drives one
 * GPU; calls on a context must be serialised by the caller.
 *
 * Reference interfaces replaced (paths inside KaiNakao/smc_inversion_fort):
 *   smcgpu_set_data            main.f90:254-307 + init.f90:5-119 (data, Sigma_SAR^-1)
 *   smcgpu_greens_batch        gfunc.f90:242-348 calc_greens_func, batched over theta
 *   smcgpu_gram_batch          smc_slip.f90:1347-1443 slip_calc_gsd_gsg, batched over theta
 *   smcgpu_fault_likelihood_batch
 *                              smc_fault.f90:66-292 fault_calc_likelihood, batched
 *                              (discretize_fault, gen_laplacian, calc_greens_func,
 *                              slip_smc_exec for every theta in one call)
 *   smcgpu_fault_smc_exec      smc_fault.f90:785-1075 fault_smc_exec
 *   smcgpu_fault_smc_exec_gsmc the same with gsmc = .true. (smc_fault.f90:9-52)
 *   smcgpu_resample_counts     smc_slip.f90:572-589 / smc_fault.f90:572-590
 *   smcgpu_qsort_              sort.cpp:3-7 qsort_ (same symbol shape)
 *   smcgpu_read_*              main.f90:107-157, init.f90:5-80 (input files)
 *   smcgpu_slip_map, smcgpu_point_cloud
 *                              main.f90:553-830 calc_slip_map, point_cloud
 */
#ifndef SMCGPU_H
#define SMCGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SMCGPU_MAX_PLANES 8

/* status codes (returned) */
#define SMCGPU_OK            0
#define SMCGPU_ERR_ARG      -1
#define SMCGPU_ERR_CUDA     -2
#define SMCGPU_ERR_NODATA   -3
#define SMCGPU_ERR_MEMORY   -4
#define SMCGPU_ERR_STATE    -5

/* per-theta status bits (status_out of the likelihood calls) */
#define SMCGPU_ST_BISECT_CAP   1   /* gamma bisection hit its iteration cap           */
#define SMCGPU_ST_STAGE_CAP    2   /* > max_stages tempering stages; neglog = 1e10    */
#define SMCGPU_ST_NONFINITE    4   /* non-finite evidence or Cholesky failure          */
#define SMCGPU_ST_NEWTON_CAP   8   /* inverse-CDF Newton loop hit 100 iterations       */
#define SMCGPU_ST_REFLECT_CAP 16   /* reflection loop hit its cap                      */
#define SMCGPU_ST_TUNE_COUNT  32   /* step-size resampling count != N                  */
#define SMCGPU_ST_WAIT_CAP    64   /* a bounded device wait (tensor-core completion)
                                      gave up; the evaluation was abandoned, neglog = 1e10 */
#define SMCGPU_ST_SNAPSHOT_IO 128   /* fault_smc_exec: a stage snapshot (<iter>.state) could
                                      not be written; the run itself is unaffected, but it
                                      cannot be resumed from that stage                 */

/* theta layouts */
#define SMCGPU_LAYOUT_TRACE          0  /* [ymin ymax (x_i y_i)_{i<nplane} dip_1..n la2 ls_sar ls_gnss] (init.f90:152-167) */
#define SMCGPU_LAYOUT_TRACE_FIXBEND  1  /* [ymin ymax y_i.. dip_1..n la2 ls_sar ls_gnss] (init.f90:135-150)              */
#define SMCGPU_LAYOUT_RECT           2  /* [x y top length width strike dip la2 (ls_sar ls_gnss)] one buried rectangle    */

/* slip bases */
#define SMCGPU_BASIS_NODAL  0  /* bilinear nodal slip, reference (gfunc.f90:158-171) */
#define SMCGPU_BASIS_PATCH  1  /* patch-constant slip                                */

/* precisions */
#define SMCGPU_PREC_FP64   0   /* FP64 everywhere, reference operation order          */
#define SMCGPU_PREC_FP32   1   /* Green's build only: FP32 arithmetic, float output    */
#define SMCGPU_PREC_MIXED  2   /* nested SMC: FP32 leapfrog, FP64 likelihood/evidence  */

/* inner SMC step engines (smcgpu_config.inner_engine) */
#define SMCGPU_ENGINE_MMA      0   /* BF16x3 mma.sync tiles, FP32 accumulate (default)  */
#define SMCGPU_ENGINE_CUDA     1   /* FP32 FMA on CUDA cores                            */
#define SMCGPU_ENGINE_TCGEN05  2   /* BF16x3 tcgen05.mma with a tensor-memory accumulator */
#define SMCGPU_ENGINE_GLOBAL   3   /* stage matrix in global memory, streamed once per
                                      leapfrog step; any slip dimension up to 1024 (FP32
                                      FMA in MIXED, FP64 FMA in FP64).  The other engines
                                      fall back to it above their own limits.           */
#define SMCGPU_ENGINE_AUTO     4   /* per slip dimension from the engine table
                                      (smcgpu_set_engine_table; the package's autotuner
                                      writes one), else MMA / CUDA cores up to their
                                      limits and the global-matrix engine above        */

typedef struct smcgpu_config {
    int32_t layout;
    int32_t basis;
    int32_t nplane;
    int32_t nxi[SMCGPU_MAX_PLANES];
    int32_t neta[SMCGPU_MAX_PLANES];
    double xbend[SMCGPU_MAX_PLANES];
    double xmin, xmax, zmin;       /* trace extent and fault bottom (km, zmin < 0)       */
    int32_t nquad;                 /* Gauss points per patch direction (reference: 2)    */
    int32_t rect_hyper;            /* LAYOUT_RECT: theta carries log sigma2 sar/gnss     */
    double alpha;                  /* medium constant (reference: 2/3)                   */
    double max_slip;               /* slip box [0, max_slip] (m)                         */
    int32_t nparticle_slip;        /* inner particles                                    */
    int32_t ntau;                  /* leapfrog steps (reference: 50)                     */
    int32_t tuning_factor;         /* every k-th parent tunes the step (reference: 5)    */
    int32_t max_stages;            /* inner stage cap (reference: 200)                   */
    double cv_inner;               /* inner weight CV target (reference: 2.0)            */
    double cv_outer;               /* outer weight CV target (reference: 0.2)            */
    double sar_corr_len;           /* InSAR covariance range km (reference: 10)          */
    int32_t precision;             /* SMCGPU_PREC_FP64 or SMCGPU_PREC_MIXED              */
    int32_t device;                /* CUDA device ordinal                                */
    int32_t max_outer_stages;      /* stop fault_smc_exec after this many stages (0: run
                                      until gamma = 1 as the reference does; < 0: only
                                      the initial evaluation of the prior sample)       */
    int32_t inner_warps;           /* CUDA-core inner SMC engine: warps per geometry
                                      particle, 1, 2, 4 or 8; 0 picks from the batch size.
                                      Results do not depend on it.                      */
    int32_t inner_engine;          /* leapfrog engine, SMCGPU_ENGINE_*.  MIXED: warp-level
                                      tensor-core MMA (default; slip dimensions <= 256,
                                      the stage matrix streamed from global memory above
                                      128), CUDA cores (<= 192), tcgen05 (<= 128), or the
                                      global-matrix engine (<= 1024; also the fallback
                                      above each engine's limit).  FP64: CUDA cores up to
                                      128, the global-matrix engine up to 1024 (or at any
                                      size with SMCGPU_ENGINE_GLOBAL).                  */
    double patch_km;               /* > 0 (LAYOUT_RECT only): a patch size; each geometry
                                      gets its own mesh, nxi = round(length / patch_km)
                                      and neta = round(width / patch_km), clamped to
                                      [2, nxi[0]] and [2, neta[0]], so one batch mixes
                                      patch counts (and slip dimensions).  0: the fixed
                                      mesh nxi[0] x neta[0] of every geometry.  With
                                      per-geometry meshes the nested evaluation and the
                                      outer SMC run as usual; the calls that return
                                      per-geometry matrices (Green's, Gram, slip
                                      populations) need a fixed mesh.                   */
} smcgpu_config;

typedef struct smcgpu_ctx smcgpu_ctx;

/* Fill *cfg with the reference's constants (one plane, nodal basis, 2x2
 * Gauss points, alpha = 2/3, ntau = 50, tuning factor 5, 200 stages, CV 2 and
 * 0.2, 10 km SAR range, FP64). */
int32_t smcgpu_default_config(smcgpu_config *cfg);

/* Create a context on cfg->device.  Replaces the allocation block of
 * main.f90:349-390; the mesh pattern is fixed here. */
int32_t smcgpu_create(const smcgpu_config *cfg, smcgpu_ctx **out);
int32_t smcgpu_destroy(smcgpu_ctx *ctx);

/* Observations in the reference's arrays (read_observation2, init.f90:24-80):
 * obs_points(2,nobs), obs_unitvec(3,nobs), obs_sigma(nobs), dvec(nobs);
 * nsar_index(npath+1) is the reference's 1-based path start table; GNSS rows
 * follow the SAR rows in triples.  Sigma_SAR^-1 (init.f90:82-119) is built
 * here in FP64.  Copies everything to the device. */
int32_t smcgpu_set_data(smcgpu_ctx *ctx, int32_t nobs, const double *obs_points, const double *obs_unitvec,
                        const double *obs_sigma, const double *dvec, int32_t npath,
                        const int32_t *nsar_index, int32_t ngnss);

/* Work on the caller's CUDA stream (cudaStream_t passed as void*); NULL
 * selects the context's own non-blocking stream; the legacy default stream is
 * selected with cudaStreamLegacy ((void*)1). */
int32_t smcgpu_set_stream(smcgpu_ctx *ctx, void *stream);

/* Dimensions: ndim_fault, D = 2*ndof (nodal) or 2*npatch, nobs, nrow_l. */
int32_t smcgpu_dims(const smcgpu_ctx *ctx, int32_t *ndim_fault, int32_t *D, int32_t *nobs, int32_t *nrow_l);

/* Diagnostic, no reference counterpart; host only, needs no GPU.  The sweep
 * schedule of the Gibbs initialisation (slip_gen_init_particles,
 * smc_slip.f90:207-263) for a configuration: the D slip components ordered by
 * level (order, 0-based) and the level starts (level_ptr, nlevel + 1 entries).
 * No two components of a level are coupled by L^T L, and every coupled
 * component j < i has a lower level than i, so a level-by-level sweep equals
 * the sequential one.  With order == NULL only *D and *nlevel are returned. */
int32_t smcgpu_gibbs_levels(const smcgpu_config *cfg, int32_t *D, int32_t *nlevel, int32_t *order,
                            int32_t *level_ptr);

/* Green's matrices for n_theta geometries: gmat(nobs, D, n_theta), the
 * reference's gmat(nobs, 2*ndof) per theta (gfunc.f90:242-348).  precision
 * SMCGPU_PREC_FP64 writes double, SMCGPU_PREC_FP32 writes float.
 * _batch takes host buffers (copies inside the call); _batch_dev takes device
 * pointers already in HBM. */
int32_t smcgpu_greens_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, int32_t precision,
                            void *gmat);
int32_t smcgpu_greens_batch_dev(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                int32_t precision, void *gmat_dev);

/* slip_calc_gsd_gsg (smc_slip.f90:1347-1443) for n_theta geometries, FP64:
 * gsgmat(D, D, n_theta) = G^T Sigma^-1 G, gsdvec(D, n_theta) = G^T Sigma^-1 d and
 * dsd(n_theta) = d^T Sigma^-1 d, with each theta's hyperparameters scaling the
 * InSAR and GNSS blocks (sigma2_sar, sigma2_gnss).  The InSAR blocks go through
 * the whitening factor of Sigma_SAR^-1 made in set_data.  Host buffers. */
int32_t smcgpu_gram_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, double *gsgmat,
                          double *gsdvec, double *dsd);

/* smcgpu_greens_batch_dev for callers that cannot allocate device memory
 * during the call: hosts that give the whole GPU memory to their own pool
 * at start-up, and stage loops that must not pay cudaMalloc/cudaFree's
 * device-wide synchronisation.  It has no counterpart in the reference.  Its
 * scratch (per-plane geometry records) is a fixed device array of 16384
 * records (2.2 MB on every GPU that loads the library), so n_theta * nplane
 * must be <= 16384, otherwise SMCGPU_ERR_ARG.  No cudaMalloc, cudaFree or
 * allocating library call is made.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) and should come before any stream
 * capture.  The address is cached per device for the life of the process:
 * after cudaDeviceReset (or any teardown of the device's primary context) it
 * is stale, so do not call this entry point again in that process.  All calls
 * share the array: calls that overlap on the GPU race. */
int32_t smcgpu_greens_batch_noalloc(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                    int32_t precision, void *gmat_dev);

/* Nested evaluation -log Z(theta) for n_theta geometries (fault_calc_likelihood,
 * smc_fault.f90:66-292).  Every evaluation draws from the Philox4x64-10 stream
 * keyed by (seed, streams[i]); status_out gets SMCGPU_ST_* bits; a stage-cap
 * hit returns neglog = 1e10 as the reference does (smc_slip.f90:1557-1560). */
int32_t smcgpu_fault_likelihood_batch(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed,
                                      const uint64_t *streams, double *neglog_out, int32_t *status_out);
int32_t smcgpu_fault_likelihood_batch_dev(smcgpu_ctx *ctx, int32_t n_theta, const double *theta_dev,
                                          uint64_t seed, const uint64_t *streams_dev, double *neglog_dev,
                                          int32_t *status_dev);

/* Diagnostic variant of smcgpu_fault_likelihood_batch (host buffers): also
 * returns the number of tempering stages per theta and the stage-by-stage
 * tempering exponent and -log evidence increment, gamma_trace /
 * inc_trace (max_stages+2, n_theta), zero past the last stage. */
int32_t smcgpu_fault_likelihood_trace(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed,
                                      const uint64_t *streams, double *neglog_out, int32_t *status_out,
                                      int32_t *nstage_out, double *gamma_trace, double *inc_trace);

/* One nested evaluation that also returns the final slip population, the
 * data behind the reference's flag_output = 1 slip file (smc_slip.f90:1632-1660):
 * particles_out(D, nparticle_slip), likelihood_out and prior_out(nparticle_slip). */
int32_t smcgpu_fault_likelihood_posterior(smcgpu_ctx *ctx, const double *theta, uint64_t seed, uint64_t stream,
                                          double *neglog_out, int32_t *status_out, double *particles_out,
                                          double *likelihood_out, double *prior_out);

/* The full outer SMC (fault_smc_exec, smc_fault.f90:785-1075) with a uniform
 * prior box range(2, ndim_fault).  particles_out(ndim_fault, nparticle) and
 * likelihood_out(nparticle) receive the final population.  When output_dir
 * is not NULL, the reference's per-stage CSV files output_dir<iter>.csv are
 * written (the name is the prefix and the stage number concatenated, as
 * trim(output_dir)//iter//".csv" in smc_fault.f90:923-936, 1054-1067; the
 * directory is created like main.f90's "mkdir -p"). */
int32_t smcgpu_fault_smc_exec(smcgpu_ctx *ctx, const double *range, int32_t nparticle, uint64_t seed,
                              const char *output_dir, double *particles_out, double *likelihood_out,
                              double *evidence_out, int32_t *nstage_out);

/* The outer SMC in GSMC mode (gsmc = .true., main.f90:313-330): the initial
 * population is drawn from q = N(qmean, qcov) and the tempering runs from q
 * to the posterior, i.e. on L - q (smc_fault.f90:9-52, 392-485, 748-771).
 * qcov_chol is the lower Cholesky factor of qcov (the reference's qcov after
 * dpotrf('L')), qcov_inv its inverse, both ndim x ndim column-major, and
 * log_qcov_det = log det qcov, as in data/qcov.dat, qcov_inv.dat and
 * log_qcov_det.dat.  range still bounds the random-walk proposals. */
int32_t smcgpu_fault_smc_exec_gsmc(smcgpu_ctx *ctx, const double *range, int32_t nparticle, uint64_t seed,
                                   const char *output_dir, const double *qmean, const double *qcov_chol,
                                   const double *qcov_inv, double log_qcov_det, double *particles_out,
                                   double *likelihood_out, double *evidence_out, int32_t *nstage_out);

/* Continue an outer SMC from the state file output_dir<k>.state that
 * fault_smc_exec(_gsmc) writes after stage k (full-precision population,
 * likelihoods, q values, gamma, evidence).  Draws are keyed by stage, so the
 * continued run equals the uninterrupted one.  The GSMC parameters are given
 * (non-NULL) exactly when the state comes from a GSMC run; nstage_out counts
 * all stages, from the original start. */
int32_t smcgpu_fault_smc_resume(smcgpu_ctx *ctx, const double *range, int32_t nparticle, uint64_t seed,
                                const char *output_dir, const char *state_path, const double *qmean,
                                const double *qcov_chol, const double *qcov_inv, double log_qcov_det,
                                double *particles_out, double *likelihood_out, double *evidence_out,
                                int32_t *nstage_out);

/* Residual-systematic resampling counts on the device (smc_slip.f90:572-589).
 * u0 is the binary128 uniform of random_number_correction_dd carried as a
 * double-double (u0_hi + u0_lo exactly).  counts match the reference's
 * binary128 recurrence bit for bit. */
int32_t smcgpu_resample_counts(smcgpu_ctx *ctx, const double *weights, int32_t n, double u0_hi, double u0_lo,
                               int32_t *counts);

/* Drop-in for sort.cpp:3-7 qsort_(arr, index, n): orders the 1-based index[]
 * by arr[index-1] descending with the same std::sort comparator. */
void smcgpu_qsort_(int32_t *arr, int32_t *index, int32_t *n);

/* ---- readers for the reference's input files (host only; no GPU needed).
 * Fortran list-directed semantics: blank/comma separated values that may
 * continue over records, r*v repeats, D exponents, .true./T/.false./F. */
#define SMCGPU_PATH_MAX 512
typedef struct smcgpu_settings {
    int32_t nplane;
    int32_t fix_xbend;                   /* logical */
    double xbend[SMCGPU_MAX_PLANES];     /* nplane-1 values */
    int32_t nparticle_fault;
    int32_t nparticle_slip;
    char observation_path[SMCGPU_PATH_MAX];
    int32_t npath;                       /* number of InSAR paths */
    char output_dir[SMCGPU_PATH_MAX];
    double max_slip;
    int32_t nxi[SMCGPU_MAX_PLANES];
    int32_t neta[SMCGPU_MAX_PLANES];
    double xmin, xmax, zmin;
    int32_t gsmc;                        /* logical */
} smcgpu_settings;

/* data/setting.dat (main.f90:107-157). */
int32_t smcgpu_read_settings(const char *path, smcgpu_settings *out);
/* The context configuration the reference derives from the settings:
 * nodal basis, trace layout with or without fixed bends, reference constants. */
int32_t smcgpu_settings_to_config(const smcgpu_settings *st, smcgpu_config *cfg);
/* read_observation1 (init.f90:5-22): number of observation rows (records
 * after the header). */
int32_t smcgpu_count_observations(const char *path, int32_t *nobs);
/* read_observation2 (init.f90:24-80): rows "x y ex ey ez dlos sigma type";
 * consecutive "InSAR*" rows of one type form a path, "GNSS" rows come in
 * station triples.  obs_points 2 x nobs, obs_unitvec 3 x nobs (column-major),
 * nsar_index npath+1 (1-based, as the reference). */
int32_t smcgpu_read_observations(const char *path, int32_t nobs, int32_t npath, double *obs_points,
                                 double *obs_unitvec, double *obs_sigma, double *dvec, int32_t *nsar_index,
                                 int32_t *nsar_total, int32_t *ngnss);
/* data/range.dat (main.f90:497-502): per parameter a label record then
 * "lower upper"; range is 2 x ndim (column-major). */
int32_t smcgpu_read_range(const char *path, int32_t ndim, double *range);
/* A plain list of n reals: one READ per value (peak_fault.dat, main.f90:430-434)
 * when one_per_record, else one list-directed READ of all n (qmean.dat,
 * qcov.dat, main.f90:313-330). */
int32_t smcgpu_read_values(const char *path, int32_t n, int32_t one_per_record, double *out);

/* slip_smc_exec's posterior dump (smc_slip.f90:1632-1660): one record per
 * particle with the two slip components of every node (0 where the node has
 * no DOF), then likelihood and prior, Fortran f12.5.  particles is D x
 * nparticle (column-major), e.g. from smcgpu_fault_likelihood_posterior. */
int32_t smcgpu_write_slip(smcgpu_ctx *ctx, const char *path, int32_t nparticle, const double *particles,
                          const double *likelihood, const double *prior);

/* ---- post-processing of sampled geometries (main.f90:553-830) */

/* calc_slip_map (main.f90:553-664) on the device: one nested evaluation per
 * theta (as fault_likelihood_batch) and the mean of its final inner
 * population, mean_slip_out(D, n_theta) in the DOF layout. */
int32_t smcgpu_slip_map(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, uint64_t seed, const uint64_t *streams,
                        double *mean_slip_out, double *neglog_out, int32_t *status_out);
/* DOF vectors (D, n) to slip_dist(2, nnode, n): zero on nodes without a DOF
 * (the patch basis is copied unchanged, D values per theta). */
int32_t smcgpu_slip_to_nodes(const smcgpu_ctx *ctx, int32_t n, const double *slip, double *slip_nodes);
/* calc_slip_map's output file: per theta the node slips (2 x nnode), f12.5. */
int32_t smcgpu_write_slip_map(smcgpu_ctx *ctx, const char *path, int32_t n, const double *mean_slip);
/* point_cloud (main.f90:666-806) on the device: every patch of every theta
 * split into nr x nr sub-points at the cell centres of [-1, 1]^2, each with
 * its global (x, y, z) and bilinearly interpolated slip (uxi, ueta, |u|).
 * slip is slip_dist(2, nnode, n_theta) (the patch basis: (D, n_theta));
 * points_out(6, nr, nr, npatch, n_theta).  The plane record (centre, strike,
 * dip, size) is calc_greens_func's (gfunc.f90:283-296). */
int32_t smcgpu_point_cloud(smcgpu_ctx *ctx, int32_t n_theta, const double *theta, const double *slip, int32_t nr,
                           double *points_out);
/* point_cloud's files: prefix//iplane (I1) per plane, records of 6 x f12.5. */
int32_t smcgpu_write_point_cloud(smcgpu_ctx *ctx, const char *prefix, int32_t n, int32_t nr, const double *points);

/* Last error message of the context (or, when ctx is NULL, of the last
 * create call or file reader on this thread). */
const char *smcgpu_last_error(const smcgpu_ctx *ctx);

/* Engine table for SMCGPU_ENGINE_AUTO (no counterpart in the reference): for
 * slip dimensions D <= dmax[k] (ascending), engine[k] (SMCGPU_ENGINE_MMA ..
 * _GLOBAL) with warps[k] warps per geometry (CUDA-core engine; 0 = from the
 * batch size).  precision: SMCGPU_PREC_FP64 or SMCGPU_PREC_MIXED; n = 0
 * clears the table.  The package's autotuner times the candidates per slip
 * dimension on the device and writes the table it loads. */
int32_t smcgpu_set_engine_table(smcgpu_ctx *ctx, int32_t precision, int32_t n, const int32_t *dmax,
                                const int32_t *engine, const int32_t *warps);

/* ---- run statistics (no counterpart in the reference, which prints only the
 * wall time of one nested evaluation, main.f90:464-480) ----
 * smcgpu_stats_reset clears the counters and turns recording on (enable != 0)
 * or off.  While on, every nested batch records device events around its
 * inner SMC launch and around the whole batch (Green's build to inner SMC),
 * and the inner kernel adds its tempering stages and HMC trajectories to two
 * device counters.  smcgpu_stats_get synchronises the context's stream and
 * returns the totals since the reset. */
typedef struct smcgpu_stats {
    int64_t nested_evals;        /* geometries evaluated                                  */
    int64_t inner_stages;        /* tempering stages, summed over evaluations             */
    int64_t inner_trajectories;  /* HMC trajectories (tuning + sampling), summed          */
    double inner_kernel_ms;      /* device time of the inner SMC launches                 */
    double nested_ms;            /* device time of the nested batches                      */
} smcgpu_stats;
int32_t smcgpu_stats_reset(smcgpu_ctx *ctx, int32_t enable);
int32_t smcgpu_stats_get(smcgpu_ctx *ctx, smcgpu_stats *out);
/* Per-stage timing of the last smcgpu_fault_smc_exec / _gsmc / _resume call
 * (always recorded, host wall clock): seconds[k] and evals[k] for k = 0 (the
 * initial population's evaluation; absent after a resume) and the stages
 * 1..nstage; up to max entries are written, *n_out gets the number recorded. */
int32_t smcgpu_outer_stage_times(smcgpu_ctx *ctx, int32_t max, double *seconds, int64_t *evals, int32_t *n_out);

#ifdef __cplusplus
}
#endif
#endif
