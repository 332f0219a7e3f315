// Host-side launchers of the device kernels (one translation unit each).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "mesh.h"

namespace smc {

// greens.cu
cudaError_t launch_planes(const MeshDev &m, int n_theta, const double *theta_dev, PlaneGeom *planes_dev,
                          cudaStream_t s);
cudaError_t launch_greens(const MeshDev &m, int n_theta, const PlaneGeom *planes_dev, int precision, void *gmat_dev,
                          cudaStream_t s);

// Per-theta prior / data-weight record produced by the setup kernel.
struct ThetaAux {
    double alpha2, log_alpha2, log_sigma_sar2, log_sigma_gnss2, sigma_sar2, sigma_gnss2;
    double lconst;  // nsar*log_sigma_sar2/2 + 3*ngnss*log_sigma_gnss2/2 (smc_slip.f90:87)
};

// setup.cu: L values (ELL), L^T values, L^T L (CSR on the fixed pattern), hyper-parameters
cudaError_t launch_setup(const MeshDev &m, int n_theta, const double *theta_dev, const PlaneGeom *planes_dev,
                         double *lval, double *ltval, double *llval, ThetaAux *aux, cudaStream_t s);

// gram.cu: A = G^T Sigma^-1 G, b = G^T Sigma^-1 d, dsd (smc_slip.f90:1347-1443)
// gw: n_theta*D*nsar work buffer for the whitened InSAR rows (unused without InSAR)
cudaError_t launch_gram(const MeshDev &m, int n_theta, const double *gmat, const double *roww, const double *dx,
                        const ThetaAux *aux, double dsd_sar, double dsd_gnss, double *A, double *b, double *dsd,
                        double *gw, cudaStream_t s);

// resample.cu
cudaError_t launch_resample_counts(const double *w, int n, double u_hi, double u_lo, int *counts, int *flag,
                                   cudaStream_t s);

// postproc.cu: mean inner population per geometry; sub-patch slip point cloud
cudaError_t launch_mean_particles(int n, int N, int D, const double *parts, double *out, cudaStream_t s);
cudaError_t launch_point_cloud(const MeshDev &m, int n, const PlaneGeom *planes, const double *slip, int slip_stride,
                               int nr, double *points, cudaStream_t s);

}  // namespace smc
