// Theta-independent fault mesh pattern (host) and the by-value kernel
// parameter block (device).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/smcgpu.h"

namespace smc {

static constexpr int MAXP = SMCGPU_MAX_PLANES;
static constexpr int MAXQ = 8;      // Gauss points per direction
static constexpr int LL_MAXNZ = 32; // structural nonzeros per row of L^T L

// Passed by value to kernels.
struct MeshDev {
    int layout, basis, nquad, rect_hyper, ndim_fault;
    int nplane, nnode, npatch, ndof, D, npt, nrow;
    int nobs, nsar, ngnss, nstation, npath;
    int nxi[MAXP], neta[MAXP], node_off[MAXP + 1], patch_off[MAXP + 1];
    double xbend[MAXP];
    double xmin, xmax, zmin, alpha;
    double gq_x[MAXQ], gq_w[MAXQ];
    // device tables (uploaded once)
    const int *dof_of_node;   // [nnode] -> dof or -1 (nodal basis)
    const int *l_col;         // [nrow*9] column of L (0-based DOF column), -1 pad
    const signed char *l_k;   // [nrow*9*3] integer multiples of 1/dxi^2, 1/deta^2, 1/(4 dxi deta)
    const int *l_plane;       // [nrow] plane of the row
    const int *lt_row;        // [D*9] rows of L in column order, -1 pad
    const signed char *lt_k;  // [D*9*3]
    const int *lt_plane;      // [D]
    const int *ll_ptr;        // [D+1] CSR of the structural pattern of L^T L
    const int *ll_col;        // [nnz]
    int ll_nnz, ll_maxrow;
    // Gibbs sweep levels: components ordered by level (gb_order), level l holding
    // gb_order[gb_lvl_ptr[l] .. gb_lvl_ptr[l+1]); no two components of a level are
    // coupled by L^T L, and every coupled earlier component has a lower level
    const int *gb_order, *gb_lvl_ptr;
    int gb_nlevel;
    // observations
    const double *st_x, *st_y;      // [nstation]
    const int *st_row, *st_nrow;    // first row, 1 (SAR) or 3 (GNSS)
    const double *obs_e;            // [nobs*3]
    const double *obs_sigma, *dvec; // [nobs]
    const int *nsar_index;          // [npath+1] zero-based
    const double *sar_inv;          // concatenated Sigma^-1 blocks
    const long long *sar_off;       // [npath] offsets into sar_inv
};

struct MeshPattern {
    int layout = 0, basis = 0, nquad = 2, rect_hyper = 0, ndim_fault = 0;
    int nplane = 1, nnode = 0, npatch = 0, ndof = 0, D = 0, npt = 0, nrow = 0;
    int nxi[MAXP] = {0}, neta[MAXP] = {0}, node_off[MAXP + 1] = {0}, patch_off[MAXP + 1] = {0};
    std::vector<int> dof_of_node, id_dof;
    std::vector<int> l_col, l_plane, lt_row, lt_plane;
    std::vector<signed char> l_k, lt_k;
    std::vector<int> ll_ptr, ll_col;
    int ll_maxrow = 0;
    std::vector<int> gb_order, gb_lvl_ptr;   // Gibbs sweep levels (see MeshDev)
    std::vector<double> gq_x, gq_w;

    // returns empty string on success
    std::string build(const smcgpu_config &cfg);
};

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w);

}  // namespace smc
