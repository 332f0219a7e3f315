/*
 * CPU oracle for the nested-SMC fault-geometry + slip inversion hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of the
 * reference Fortran (KaiNakao/smc_inversion_fort, src/*.f90, src/sort.cpp)
 * used as the checker for the CUDA path and as the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference legs may load it.  The product library never links it.
 *
 * Parity status: the reference ships no tests, fixtures or golden vectors
 * and cannot be compiled here (no Fortran compiler, MPI or MKL), so the
 * restatement is pinned by (1) an independent 50-digit mpmath evaluation of
 * Okada's point-source formulas, (2) linearity / symmetry identities,
 * (3) a finite-difference check of the slip gradient, (4) binary128
 * resampling known-answer vectors generated by the committed script in
 * tests/golden/, and (5) numpy's Philox4x64-10 bit generator for the
 * random stream.  The random stream itself is a replacement for the Fortran
 * intrinsic random_number, so posterior parity with the reference binary is
 * statistical, not bitwise.
 */
#ifndef SMC_ORACLE_H
#define SMC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_PLANES 8

typedef struct orc_setup {
    int32_t layout;      /* 0 trace polyline (fix_xbend=.false.), 1 trace with fixed x-bends, 2 buried rectangle */
    int32_t basis;       /* 0 nodal bilinear (reference), 1 patch-constant */
    int32_t nplane;
    int32_t nxi[ORC_MAX_PLANES];
    int32_t neta[ORC_MAX_PLANES];
    double xbend[ORC_MAX_PLANES];
    double xmin, xmax, zmin;
    int32_t nquad;       /* Gauss points per patch direction; 2 in the reference */
    int32_t rect_hyper;  /* layout 2: 1 -> theta also carries log sigma2_sar, log sigma2_gnss */
    double alpha;        /* medium constant (lambda+mu)/(lambda+2mu); 2/3 in the reference */
    double max_slip;
    int32_t nparticle_slip;
    int32_t ntau;        /* leapfrog steps (50 in the reference) */
    int32_t tuning_factor;
    int32_t max_stages;  /* 200 in the reference */
    double cv_inner;     /* 2.0 */
    double cv_outer;     /* 0.2 */
    int32_t nobs, nsar_total, ngnss, npath;
    const int32_t *nsar_index;   /* npath+1 zero-based row offsets */
    const double *obs_points;    /* [nobs][2]  (x, y) km */
    const double *obs_unitvec;   /* [nobs][3]  line-of-sight unit vectors */
    const double *obs_sigma;     /* [nobs] cm */
    const double *dvec;          /* [nobs] cm */
    const double *sigma_sar_inv; /* concatenated per path, nsar_p x nsar_p column-major */
    int32_t max_outer_stages;    /* 0: until gamma = 1; < 0: initial evaluation only; k: k stages */
} orc_setup;

typedef struct orc_dims_t {
    int32_t ndim_fault, D, nnode, ndof, npatch, nrow_l;
} orc_dims_t;

/* status bits shared with the CUDA path (same meaning) */
#define ORC_ST_BISECT_CAP   1
#define ORC_ST_STAGE_CAP    2
#define ORC_ST_NONFINITE    4
#define ORC_ST_NEWTON_CAP   8
#define ORC_ST_REFLECT_CAP 16
#define ORC_ST_TUNE_COUNT  32

void orc_philox4x64(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]);
double orc_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, uint64_t i, uint64_t j);
double orc_normal(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, uint64_t i, uint64_t d);
void orc_quad_uniform(uint64_t seed, uint64_t stream, uint32_t purpose, uint32_t stage, double *hi, double *lo);

int orc_dims(const orc_setup *s, orc_dims_t *out);
void orc_dc3d0(double alpha, double x, double y, double z, double depth, double dip,
               double pot1, double pot2, double pot3, double pot4, double u[12], int32_t *iret);
void orc_plane_params(const orc_setup *s, const double *theta, double *out /* nplane x 7 */);
int orc_greens(const orc_setup *s, const double *theta, double *gmat /* nobs x D col-major */);
int orc_laplacian(const orc_setup *s, const double *theta, int32_t *lidx, double *lval,
                  int32_t *ltidx, double *ltval, double *llmat);
void orc_sigma_sar_inv(int32_t nobs, int32_t npath, const int32_t *nsar_index, const double *obs_points,
                       const double *obs_sigma, double corr_len, double *out);
void orc_gram(const orc_setup *s, const double *gmat, double sigma_sar2, double sigma_gnss2,
              double *gsgmat, double *gsdvec, double *dsd);
void orc_hyper(const orc_setup *s, const double *theta, double *log_alpha2,
               double *log_sigma_sar2, double *log_sigma_gnss2);

typedef struct orc_inner_trace {
    int32_t nstage;
    double *gamma;       /* max_stages+1 */
    double *neglog_inc;  /* max_stages+1 */
    int32_t *assigned;   /* optional: (max_stages+1) x N */
} orc_inner_trace;

int orc_fault_likelihood(const orc_setup *s, const double *theta, uint64_t seed, uint64_t stream,
                         double *neglog, double *particles /* optional N x D */,
                         double *likelihood /* optional N */, double *prior /* optional N */,
                         orc_inner_trace *trace /* optional */);
// likelihood, prior and tempered gradient gamma dL/dx + dP/dx at one slip vector (returns D)
int orc_slip_energy(const orc_setup *s, const double *theta, double gamma, const double *x, double *lik, double *pri,
                    double *grad);
int orc_fault_likelihood_batch(const orc_setup *s, int32_t n, const double *theta, uint64_t seed,
                               const uint64_t *streams, double *neglog, int32_t *status, int32_t nthreads);
int orc_greens_batch(const orc_setup *s, int32_t n, const double *theta, double *gmat, int32_t nthreads);

void orc_resample(const double *w, int32_t n, double u_hi, double u_lo, int32_t *counts);
void orc_qsort_(int32_t *arr, int32_t *index, int32_t *n);

/* point_cloud (main.f90:666-781): sub-points of every patch with global
 * coordinates and interpolated slip; slip is slip_dist(2, nnode) (nodal) or
 * the D patch values; points [npatch][nr][nr][6] = x, y, z, uxi, ueta, |u| */
int orc_point_cloud(const orc_setup *s, const double *theta, const double *slip, int32_t nr, double *points);

/* GSMC reference distribution q = N(qmean, qcov) of the outer SMC
 * (smc_fault.f90:9-27, 41-52; main.f90:313-330) */
typedef struct orc_gsmc {
    const double *qmean;      /* [ndim] */
    const double *qcov_chol;  /* [ndim][ndim] lower Cholesky factor of qcov, column-major */
    const double *qcov_inv;   /* [ndim][ndim] column-major */
    double log_qcov_det;
} orc_gsmc;

int orc_fault_smc(const orc_setup *s, const double *range /* [ndim][2] */, int32_t nparticle,
                  int32_t numprocs, uint64_t seed, int32_t nthreads, double *particles_out,
                  double *likelihood_out, double *evidence_out, int32_t *nstage_out,
                  double *gamma_out /* optional, 1024 */, const orc_gsmc *gsmc /* NULL: uniform prior */);

#ifdef __cplusplus
}
#endif
#endif
