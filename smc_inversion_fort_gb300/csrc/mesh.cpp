// Theta-independent mesh pattern: node / patch numbering and DOF table of
// discretize_fault (init.f90:198-293, main.f90:209-246), and the sparsity
// pattern of the smoothing operator of gen_laplacian / gen_sparse_lmat
// (init.f90:295-521).  Only the pattern is fixed here; the entry values
// depend on theta through the per-plane spacings dxi, deta and are
// evaluated on the device from the integer multiples stored below.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <set>

namespace smc {

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    if (n == 2) {  // the reference's literal +-1/sqrt(3) (gfunc.f90:125-128)
        x[0] = -1.0 / std::sqrt(3.0);
        x[1] = 1.0 / std::sqrt(3.0);
        w[0] = w[1] = 1.0;
        return;
    }
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < n; ++i) {
        long double z = std::cos(pi * (i + 0.75L) / (n + 0.5L)), dp = 1;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1, p2 = 0;
            for (int k = 1; k <= n; ++k) {
                long double p3 = p2;
                p2 = p1;
                p1 = ((2 * k - 1) * z * p2 - (k - 1) * p3) / k;
            }
            dp = n * (z * p1 - p2) / (z * z - 1);
            long double z1 = z;
            z = z1 - p1 / dp;
            if (std::fabs((double)(z - z1)) < 1e-19) break;
        }
        x[n - 1 - i] = (double)z;
        w[n - 1 - i] = (double)(2 / ((1 - z * z) * dp * dp));
    }
}

namespace {
struct K3 { int kx = 0, ky = 0, kc = 0; };
}

std::string MeshPattern::build(const smcgpu_config &cfg) {
    layout = cfg.layout;
    basis = cfg.basis;
    nquad = cfg.nquad;
    rect_hyper = cfg.rect_hyper;
    nplane = cfg.nplane;
    if (nplane < 1 || nplane > MAXP) return "nplane out of range";
    if (layout < 0 || layout > 2) return "unknown theta layout";
    if (basis < 0 || basis > 1) return "unknown slip basis";
    if (layout == SMCGPU_LAYOUT_RECT && nplane != 1) return "the rectangle layout has one plane";
    if (nquad < 1 || nquad > MAXQ) return "nquad out of range";
    if (layout == 0) ndim_fault = 3 * nplane + 3;
    else if (layout == 1) ndim_fault = 2 * nplane + 4;
    else ndim_fault = rect_hyper ? 10 : 8;
    nnode = npatch = 0;
    int npt_tot = 0;
    for (int ip = 0; ip < nplane; ++ip) {
        nxi[ip] = cfg.nxi[ip];
        neta[ip] = cfg.neta[ip];
        if (nxi[ip] < 2 || neta[ip] < 2) return "each plane needs nxi >= 2 and neta >= 2";
        node_off[ip] = nnode;
        patch_off[ip] = npatch;
        nnode += (nxi[ip] + 1) * (neta[ip] + 1);
        npatch += nxi[ip] * neta[ip];
    }
    node_off[nplane] = nnode;
    patch_off[nplane] = npatch;
    // DOF table (init.f90:250-265)
    dof_of_node.assign(nnode, -1);
    id_dof.clear();
    for (int ip = 0; ip < nplane; ++ip)
        for (int j = 0; j <= neta[ip]; ++j)
            for (int i = 0; i <= nxi[ip]; ++i) {
                int node = node_off[ip] + i + (nxi[ip] + 1) * j;
                if (j == 0) continue;
                if (ip == 0 && i == 0) continue;
                if (ip == nplane - 1 && i == nxi[ip]) continue;
                dof_of_node[node] = (int)id_dof.size();
                id_dof.push_back(node);
            }
    ndof = (int)id_dof.size();
    D = basis == SMCGPU_BASIS_NODAL ? 2 * ndof : 2 * npatch;

    // Smoothing stencil on the point grid of each plane (nodes or patch
    // centres), as integer multiples of the three step terms.
    std::vector<int> px(nplane), py(nplane), poff(nplane + 1);
    for (int ip = 0; ip < nplane; ++ip) {
        px[ip] = basis == SMCGPU_BASIS_NODAL ? nxi[ip] + 1 : nxi[ip];
        py[ip] = basis == SMCGPU_BASIS_NODAL ? neta[ip] + 1 : neta[ip];
        poff[ip] = npt_tot;
        npt_tot += px[ip] * py[ip];
    }
    poff[nplane] = npt_tot;
    npt = npt_tot;
    nrow = 2 * npt;
    std::vector<std::map<int, K3>> lu(npt);
    std::vector<int> plane_of_pt(npt);
    for (int ip = 0; ip < nplane; ++ip) {
        int nx = px[ip] - 1, ny = py[ip] - 1, W = nx + 1, off = poff[ip];
        for (int in1 = off + 1; in1 <= off + (nx + 1) * (ny + 1); ++in1) {
            int k = (in1 - 1 - off) % (nx + 1) + 1;
            int l = (in1 - 1 - off) / (nx + 1) + 1;
            int in = in1 - 1;
            plane_of_pt[in] = ip;
            auto &r = lu[in];
            r[in].kx -= 2;
            if (k == nx + 1) r[in - 1].kx += 1; else r[in + 1].kx += 1;
            if (k == 1) r[in + 1].kx += 1; else r[in - 1].kx += 1;
            if (l == ny + 1) r[in - W].ky += 1; else r[in + W].ky += 1;
            if (l == 1) r[in + W].ky += 1; else r[in - W].ky += 1;
            if (k == nx + 1 && l == ny + 1) r[in - W - 1].kc += 1;
            else if (k == nx + 1) r[in + W - 1].kc += 1;
            else if (l == ny + 1) r[in - W + 1].kc += 1;
            else r[in + W + 1].kc += 1;
            if (k == 1 && l == ny + 1) r[in - W + 1].kc -= 1;
            else if (k == 1) r[in + W + 1].kc -= 1;
            else if (l == ny + 1) r[in - W - 1].kc -= 1;
            else r[in + W - 1].kc -= 1;
            if (k == 1 && l == 1) r[in + W + 1].kc += 1;
            else if (k == 1) r[in - W + 1].kc += 1;
            else if (l == 1) r[in + W - 1].kc += 1;
            else r[in - W - 1].kc += 1;
            if (k == nx + 1 && l == 1) r[in + W - 1].kc -= 1;
            else if (k == nx + 1) r[in - W - 1].kc -= 1;
            else if (l == 1) r[in + W + 1].kc -= 1;
            else r[in - W + 1].kc -= 1;
        }
    }
    // DOF columns of the point grid
    std::vector<int> dof_of_pt(npt, -1);
    if (basis == SMCGPU_BASIS_NODAL) {
        for (int d = 0; d < ndof; ++d) dof_of_pt[id_dof[d]] = d;
    } else {
        for (int i = 0; i < npt; ++i) dof_of_pt[i] = i;
    }
    // L = two-component expansion: row 2*in+c, column 2*dof(jn)+c
    l_col.assign((size_t)nrow * 9, -1);
    l_k.assign((size_t)nrow * 9 * 3, 0);
    l_plane.assign(nrow, 0);
    std::vector<std::vector<std::pair<int, K3>>> cols(D);
    for (int in = 0; in < npt; ++in) {
        std::vector<std::pair<int, K3>> ent;
        for (auto &kv : lu[in]) {
            const K3 &k = kv.second;
            if (k.kx == 0 && k.ky == 0 && k.kc == 0) continue;
            int d = dof_of_pt[kv.first];
            if (d < 0) continue;
            if ((k.kx != 0) + (k.ky != 0) + (k.kc != 0) > 1) return "mixed stencil entry";
            ent.push_back({d, k});
        }
        std::sort(ent.begin(), ent.end(), [](const std::pair<int, K3> &a, const std::pair<int, K3> &b) { return a.first < b.first; });
        if (ent.size() > 9) return "more than 9 stencil entries in a row";
        for (int c = 0; c < 2; ++c) {
            int row = 2 * in + c;
            l_plane[row] = plane_of_pt[in];
            for (size_t q = 0; q < ent.size(); ++q) {
                int col = 2 * ent[q].first + c;
                l_col[(size_t)row * 9 + q] = col;
                l_k[((size_t)row * 9 + q) * 3 + 0] = (signed char)ent[q].second.kx;
                l_k[((size_t)row * 9 + q) * 3 + 1] = (signed char)ent[q].second.ky;
                l_k[((size_t)row * 9 + q) * 3 + 2] = (signed char)ent[q].second.kc;
                cols[col].push_back({row, ent[q].second});
            }
        }
    }
    lt_row.assign((size_t)D * 9, -1);
    lt_k.assign((size_t)D * 9 * 3, 0);
    lt_plane.assign(D, 0);
    for (int c = 0; c < D; ++c) {
        auto &v = cols[c];
        std::sort(v.begin(), v.end(), [](const std::pair<int, K3> &a, const std::pair<int, K3> &b) { return a.first < b.first; });
        if (v.size() > 9) return "more than 9 entries in a column of L";
        for (size_t q = 0; q < v.size(); ++q) {
            lt_row[(size_t)c * 9 + q] = v[q].first;
            lt_k[((size_t)c * 9 + q) * 3 + 0] = (signed char)v[q].second.kx;
            lt_k[((size_t)c * 9 + q) * 3 + 1] = (signed char)v[q].second.ky;
            lt_k[((size_t)c * 9 + q) * 3 + 2] = (signed char)v[q].second.kc;
        }
        lt_plane[c] = v.empty() ? 0 : l_plane[v[0].first];
    }
    // structural pattern of L^T L
    ll_ptr.assign(D + 1, 0);
    ll_col.clear();
    ll_maxrow = 0;
    for (int i = 0; i < D; ++i) {
        std::set<int> js;
        for (auto &e : cols[i]) {
            int row = e.first;
            for (int q = 0; q < 9; ++q) {
                int c = l_col[(size_t)row * 9 + q];
                if (c >= 0) js.insert(c);
            }
        }
        for (int j : js) ll_col.push_back(j);
        ll_ptr[i + 1] = (int)ll_col.size();
        ll_maxrow = std::max(ll_maxrow, (int)js.size());
    }
    if (ll_maxrow > LL_MAXNZ) return "L^T L row longer than LL_MAXNZ";
    // levels of the Gibbs sweep (slip_gen_init_particles, smc_slip.f90:207-263):
    // component i is updated after every coupled component j < i and before
    // every coupled j > i; level(i) = 1 + max level of its coupled j < i, so
    // updating level by level, the components of one level in any order,
    // reproduces the sequential sweep exactly
    {
        std::vector<int> level(D, 0);
        int nlevel = D > 0 ? 1 : 0;
        for (int i = 0; i < D; ++i) {
            for (int e = ll_ptr[i]; e < ll_ptr[i + 1]; ++e)
                if (ll_col[e] < i) level[i] = std::max(level[i], level[ll_col[e]] + 1);
            nlevel = std::max(nlevel, level[i] + 1);
        }
        gb_lvl_ptr.assign(nlevel + 1, 0);
        for (int i = 0; i < D; ++i) ++gb_lvl_ptr[level[i] + 1];
        for (int l = 0; l < nlevel; ++l) gb_lvl_ptr[l + 1] += gb_lvl_ptr[l];
        gb_order.assign(D, 0);
        std::vector<int> fill(gb_lvl_ptr.begin(), gb_lvl_ptr.end() - 1);
        for (int i = 0; i < D; ++i) gb_order[fill[level[i]]++] = i;
    }
    gauss_legendre(nquad, gq_x, gq_w);
    return "";
}

}  // namespace smc
