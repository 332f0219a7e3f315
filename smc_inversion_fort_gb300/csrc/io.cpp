// Readers for the reference's input files, so that an unchanged reference
// run directory drives the GPU path:
//   setting.dat          main.f90:107-157
//   observation file     init.f90:5-80 (read_observation1 / read_observation2)
//   range.dat            main.f90:497-502 (prior box of the outer SMC)
//   peak_fault.dat, qmean.dat ...  main.f90:313-330, 430-434 (plain value lists)
//
// The files are read with Fortran list-directed semantics: values separated by
// blanks or commas, a value list may continue over several records, every
// READ statement consumes at least one record, "r*v" repeats v r times, "/"
// ends the list, D exponents are accepted, logicals are .true./T/.false./F,
// and an "(a)" read takes the whole record.
#include <sys/stat.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "context.h"

namespace smc {

std::string fortran_f(double v, int w, int d) {
    char buf[512];
    if (std::isnan(v)) {
        snprintf(buf, sizeof buf, "%*s", w, "NaN");
    } else if (std::isinf(v)) {
        snprintf(buf, sizeof buf, "%*s", w, v < 0 ? "-Infinity" : "Infinity");
    } else {
        snprintf(buf, sizeof buf, "%*.*f", w, d, v);
    }
    if ((int)strlen(buf) > w) return std::string((size_t)w, '*');
    return buf;
}

void mkdir_p(const std::string &path) {
    for (size_t i = 1; i <= path.size(); ++i)
        if (i == path.size() || path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

}  // namespace smc

namespace {

struct ListReader {
    std::vector<std::string> rec;
    size_t next = 0;
    std::string err;

    bool open(const char *path) {
        std::ifstream f(path);
        if (!f) { err = std::string("cannot open ") + path; return false; }
        std::string line;
        while (std::getline(f, line)) {
            if (!line.empty() && line.back() == '\r') line.pop_back();
            rec.push_back(line);
        }
        return true;
    }
    bool eof() const { return next >= rec.size(); }

    // split one record into list-directed items (repeat counts expanded)
    static bool items(const std::string &s, std::vector<std::string> &out, bool &slash) {
        size_t i = 0, n = s.size();
        slash = false;
        while (i < n) {
            while (i < n && (s[i] == ' ' || s[i] == '\t' || s[i] == ',')) ++i;
            if (i >= n) break;
            if (s[i] == '/') { slash = true; return true; }
            std::string tok;
            if (s[i] == '\'' || s[i] == '"') {
                char q = s[i++];
                while (i < n) {
                    if (s[i] == q) {
                        if (i + 1 < n && s[i + 1] == q) { tok += q; i += 2; continue; }
                        ++i;
                        break;
                    }
                    tok += s[i++];
                }
            } else {
                while (i < n && s[i] != ' ' && s[i] != '\t' && s[i] != ',' && s[i] != '/') tok += s[i++];
            }
            size_t star = tok.find('*');
            if (star != std::string::npos && star > 0 &&
                tok.find_first_not_of("0123456789") == star) {
                int r = atoi(tok.substr(0, star).c_str());
                std::string v = tok.substr(star + 1);
                for (int k = 0; k < r; ++k) out.push_back(v);
            } else {
                out.push_back(tok);
            }
        }
        return true;
    }

    // one list-directed READ of n items; consumes whole records
    bool read_items(size_t n, std::vector<std::string> &out) {
        out.clear();
        if (eof()) { err = "unexpected end of file"; return false; }
        do {
            if (eof()) { err = "unexpected end of file"; return false; }
            bool slash = false;
            items(rec[next++], out, slash);
            if (slash) break;
        } while (out.size() < n);
        if (out.size() < n) { err = "too few values"; return false; }
        out.resize(n);
        return true;
    }
    bool skip() {
        if (eof()) { err = "unexpected end of file"; return false; }
        ++next;
        return true;
    }
    bool read_line(std::string &s) {
        if (eof()) { err = "unexpected end of file"; return false; }
        s = rec[next++];
        size_t b = s.find_first_not_of(" \t"), e = s.find_last_not_of(" \t");
        s = b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
        return true;
    }
    static bool to_double(const std::string &t, double &v) {
        std::string u = t;
        for (char &c : u)
            if (c == 'd' || c == 'D') c = 'e';
        char *end = nullptr;
        v = strtod(u.c_str(), &end);
        return !u.empty() && end && *end == '\0';
    }
    static bool to_int(const std::string &t, int &v) {
        char *end = nullptr;
        long x = strtol(t.c_str(), &end, 10);
        v = (int)x;
        return !t.empty() && end && *end == '\0';
    }
    static bool to_logical(const std::string &t, int &v) {
        size_t i = (!t.empty() && t[0] == '.') ? 1 : 0;
        if (i >= t.size()) return false;
        char c = (char)toupper((unsigned char)t[i]);
        if (c == 'T') { v = 1; return true; }
        if (c == 'F') { v = 0; return true; }
        return false;
    }
    bool doubles(size_t n, double *out) {
        std::vector<std::string> it;
        if (!read_items(n, it)) return false;
        for (size_t k = 0; k < n; ++k)
            if (!to_double(it[k], out[k])) { err = "bad real value '" + it[k] + "'"; return false; }
        return true;
    }
    bool ints(size_t n, int *out) {
        std::vector<std::string> it;
        if (!read_items(n, it)) return false;
        for (size_t k = 0; k < n; ++k)
            if (!to_int(it[k], out[k])) { err = "bad integer value '" + it[k] + "'"; return false; }
        return true;
    }
    bool logical(int &v) {
        std::vector<std::string> it;
        if (!read_items(1, it)) return false;
        if (!to_logical(it[0], v)) { err = "bad logical value '" + it[0] + "'"; return false; }
        return true;
    }
    // list-directed read of one character item (read_observation1's counter)
    bool any_item() {
        while (!eof()) {
            std::vector<std::string> it;
            bool slash = false;
            items(rec[next++], it, slash);
            if (!it.empty() || slash) return true;
        }
        return false;
    }
};

int fail(const std::string &where, const std::string &msg) {
    smc::g_create_err = where + ": " + msg;
    return SMCGPU_ERR_ARG;
}

void copy_path(char *dst, const std::string &s) {
    size_t n = std::min(s.size(), (size_t)SMCGPU_PATH_MAX - 1);
    memcpy(dst, s.data(), n);
    dst[n] = '\0';
}

}  // namespace

extern "C" int32_t smcgpu_read_settings(const char *path, smcgpu_settings *out) {
    smc::g_create_err.clear();
    if (!path || !out) return fail("read_settings", "null argument");
    memset(out, 0, sizeof(*out));
    ListReader r;
    if (!r.open(path)) return fail("read_settings", r.err);
    std::string s;
    int v = 0;
#define RD(x)                                                                   \
    do {                                                                        \
        if (!(x)) return fail(std::string("read_settings ") + path, r.err);     \
    } while (0)
    RD(r.skip());                      // number of fault planes
    RD(r.ints(1, &out->nplane));
    if (out->nplane < 1 || out->nplane > SMCGPU_MAX_PLANES)
        return fail("read_settings", "nplane must be 1.." + std::to_string(SMCGPU_MAX_PLANES));
    RD(r.skip());                      // fix-xbend
    RD(r.logical(v));
    out->fix_xbend = v;
    RD(r.skip());                      // xbend (nplane-1 values; the record is consumed even when empty)
    RD(r.doubles((size_t)out->nplane - 1, out->xbend));
    RD(r.skip());
    RD(r.skip());                      // number of samples for fault
    RD(r.ints(1, &out->nparticle_fault));
    RD(r.skip());                      // number of samples for slip
    RD(r.ints(1, &out->nparticle_slip));
    RD(r.skip());
    RD(r.skip());                      // observation path
    RD(r.read_line(s));
    copy_path(out->observation_path, s);
    RD(r.skip());                      // number of SAR paths
    RD(r.ints(1, &out->npath));
    RD(r.skip());                      // output directory path
    RD(r.read_line(s));
    copy_path(out->output_dir, s);
    RD(r.skip());
    RD(r.skip());                      // max slip (m)
    RD(r.doubles(1, &out->max_slip));
    RD(r.skip());
    RD(r.skip());                      // nxi
    RD(r.ints((size_t)out->nplane, out->nxi));
    RD(r.skip());                      // neta
    RD(r.ints((size_t)out->nplane, out->neta));
    RD(r.skip());
    RD(r.skip());                      // xmin
    RD(r.doubles(1, &out->xmin));
    RD(r.skip());                      // xmax
    RD(r.doubles(1, &out->xmax));
    RD(r.skip());                      // zmin
    RD(r.doubles(1, &out->zmin));
    RD(r.skip());
    RD(r.skip());                      // GSMC
    RD(r.logical(v));
    out->gsmc = v;
#undef RD
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_settings_to_config(const smcgpu_settings *st, smcgpu_config *cfg) {
    if (!st || !cfg) return SMCGPU_ERR_ARG;
    smcgpu_default_config(cfg);
    cfg->layout = st->fix_xbend ? SMCGPU_LAYOUT_TRACE_FIXBEND : SMCGPU_LAYOUT_TRACE;
    cfg->basis = SMCGPU_BASIS_NODAL;
    cfg->nplane = st->nplane;
    for (int i = 0; i < SMCGPU_MAX_PLANES; ++i) {
        cfg->nxi[i] = i < st->nplane ? st->nxi[i] : 0;
        cfg->neta[i] = i < st->nplane ? st->neta[i] : 0;
        cfg->xbend[i] = i < st->nplane - 1 ? st->xbend[i] : 0.0;
    }
    cfg->xmin = st->xmin;
    cfg->xmax = st->xmax;
    cfg->zmin = st->zmin;
    cfg->max_slip = st->max_slip;
    cfg->nparticle_slip = st->nparticle_slip;
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_count_observations(const char *path, int32_t *nobs) {
    smc::g_create_err.clear();
    if (!path || !nobs) return fail("count_observations", "null argument");
    ListReader r;
    if (!r.open(path)) return fail("count_observations", r.err);
    int n = -1;   // the header record is not an observation
    while (r.any_item()) ++n;
    *nobs = n;
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_read_observations(const char *path, int32_t nobs, int32_t npath, double *obs_points,
                                            double *obs_unitvec, double *obs_sigma, double *dvec,
                                            int32_t *nsar_index, int32_t *nsar_total, int32_t *ngnss) {
    smc::g_create_err.clear();
    if (!path || nobs < 0 || npath < 0 || (nobs > 0 && (!obs_points || !obs_unitvec || !obs_sigma || !dvec)) ||
        !nsar_index || !nsar_total || !ngnss)
        return fail("read_observations", "bad arguments");
    ListReader r;
    if (!r.open(path)) return fail("read_observations", r.err);
    if (!r.any_item()) return fail("read_observations", "empty file");
    std::vector<int> nsar_ls((size_t)std::max(npath, 1), 0);
    int ipath = 0, gnss_rows = 0;
    std::string type_prev;
    for (int i = 0; i < nobs; ++i) {
        std::vector<std::string> it;
        if (!r.read_items(8, it)) return fail("read_observations", "row " + std::to_string(i + 1) + ": " + r.err);
        double v[7];
        for (int k = 0; k < 7; ++k)
            if (!ListReader::to_double(it[k], v[k]))
                return fail("read_observations", "row " + std::to_string(i + 1) + ": bad value '" + it[k] + "'");
        obs_points[2 * i] = v[0];
        obs_points[2 * i + 1] = v[1];
        obs_unitvec[3 * i] = v[2];
        obs_unitvec[3 * i + 1] = v[3];
        obs_unitvec[3 * i + 2] = v[4];
        dvec[i] = v[5];
        obs_sigma[i] = v[6];
        std::string type = it[7].substr(0, 20);   // character(20)
        if (i == 0) type_prev = type;
        if (type.compare(0, 5, "InSAR") == 0) {
            if (type != type_prev) {
                ++ipath;
                if (ipath >= npath) return fail("read_observations", "more InSAR paths than npath");
                nsar_ls[ipath] = 1;
            } else {
                if (npath < 1) return fail("read_observations", "InSAR rows but npath = 0");
                nsar_ls[ipath] += 1;
            }
            type_prev = type;
        }
        if (type == "GNSS") ++gnss_rows;
    }
    nsar_index[0] = 1;
    int tot = 0;
    for (int p = 0; p < npath; ++p) {
        tot += nsar_ls[p];
        nsar_index[p + 1] = nsar_index[p] + nsar_ls[p];
    }
    *nsar_total = tot;
    *ngnss = gnss_rows / 3;
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_read_range(const char *path, int32_t ndim, double *range) {
    smc::g_create_err.clear();
    if (!path || ndim < 1 || !range) return fail("read_range", "bad arguments");
    ListReader r;
    if (!r.open(path)) return fail("read_range", r.err);
    std::string label;
    for (int i = 0; i < ndim; ++i) {
        if (!r.read_line(label) || !r.doubles(2, range + 2 * i))
            return fail("read_range", "parameter " + std::to_string(i + 1) + ": " + r.err);
    }
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_read_values(const char *path, int32_t n, int32_t one_per_record, double *out) {
    smc::g_create_err.clear();
    if (!path || n < 0 || (n > 0 && !out)) return fail("read_values", "bad arguments");
    ListReader r;
    if (!r.open(path)) return fail("read_values", r.err);
    if (one_per_record) {
        for (int i = 0; i < n; ++i)
            if (!r.doubles(1, out + i)) return fail("read_values", "value " + std::to_string(i + 1) + ": " + r.err);
    } else if (n > 0 && !r.doubles((size_t)n, out)) {
        return fail("read_values", r.err);
    }
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_write_slip(smcgpu_ctx *ctx, const char *path, int32_t nparticle, const double *particles,
                                     const double *likelihood, const double *prior) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!path || nparticle < 0 || (nparticle > 0 && (!particles || !likelihood || !prior)))
        return ctx->fail(SMCGPU_ERR_ARG, "write_slip: bad arguments");
    const smc::MeshPattern &m = ctx->mesh;
    FILE *f = std::fopen(path, "w");
    if (!f) return ctx->fail(SMCGPU_ERR_ARG, std::string("write_slip: cannot open ") + path);
    // slip_smc_exec's output (smc_slip.f90:1632-1660): per particle the two
    // slip components of every node (zero where the node carries no DOF; the
    // patch basis writes its patches), then likelihood and prior, all f12.5
    const int D = m.D;
    const bool nodal = ctx->cfg.basis == SMCGPU_BASIS_NODAL;
    const int nunit = nodal ? m.nnode : D / 2;
    std::vector<double> slip((size_t)2 * nunit);
    std::string line;
    for (int ip = 0; ip < nparticle; ++ip) {
        const double *x = particles + (size_t)ip * D;
        std::fill(slip.begin(), slip.end(), 0.0);
        if (nodal) {
            for (int idof = 0; idof < (int)m.id_dof.size(); ++idof) {
                const int inode = m.id_dof[idof];
                slip[2 * (size_t)inode] = x[2 * idof];
                slip[2 * (size_t)inode + 1] = x[2 * idof + 1];
            }
        } else {
            for (int k = 0; k < D; ++k) slip[k] = x[k];
        }
        line.clear();
        for (double v : slip) line += smc::fortran_f(v, 12, 5);
        line += smc::fortran_f(likelihood[ip], 12, 5);
        line += smc::fortran_f(prior[ip], 12, 5);
        line += '\n';
        std::fputs(line.c_str(), f);
    }
    std::fclose(f);
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_slip_to_nodes(const smcgpu_ctx *ctx, int32_t n, const double *slip, double *slip_nodes) {
    if (!ctx || n < 0 || (n > 0 && (!slip || !slip_nodes))) return SMCGPU_ERR_ARG;
    // slip_dist(2, nnode) of a DOF vector (smc_slip.f90:1645-1649): zero on
    // nodes without a DOF; the patch basis keeps its patch values
    const smc::MeshPattern &m = ctx->mesh;
    const bool nodal = ctx->cfg.basis == SMCGPU_BASIS_NODAL;
    const int out_n = nodal ? 2 * m.nnode : m.D;
    for (int t = 0; t < n; ++t) {
        const double *x = slip + (size_t)t * m.D;
        double *o = slip_nodes + (size_t)t * out_n;
        if (!nodal) {
            for (int k = 0; k < m.D; ++k) o[k] = x[k];
            continue;
        }
        for (int k = 0; k < out_n; ++k) o[k] = 0.0;
        for (int idof = 0; idof < (int)m.id_dof.size(); ++idof) {
            o[2 * (size_t)m.id_dof[idof]] = x[2 * idof];
            o[2 * (size_t)m.id_dof[idof] + 1] = x[2 * idof + 1];
        }
    }
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_write_slip_map(smcgpu_ctx *ctx, const char *path, int32_t n, const double *mean_slip) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!path || n < 0 || (n > 0 && !mean_slip)) return ctx->fail(SMCGPU_ERR_ARG, "write_slip_map: bad arguments");
    // calc_slip_map's file (main.f90:640-664): per geometry the two slip
    // components of every node, f12.5, then an end of record
    const smc::MeshPattern &m = ctx->mesh;
    const int out_n = ctx->cfg.basis == SMCGPU_BASIS_NODAL ? 2 * m.nnode : m.D;
    std::vector<double> nodes((size_t)out_n);
    FILE *f = std::fopen(path, "w");
    if (!f) return ctx->fail(SMCGPU_ERR_ARG, std::string("write_slip_map: cannot open ") + path);
    std::string line;
    for (int t = 0; t < n; ++t) {
        smcgpu_slip_to_nodes(ctx, 1, mean_slip + (size_t)t * m.D, nodes.data());
        line.clear();
        for (double v : nodes) line += smc::fortran_f(v, 12, 5);
        line += '\n';
        std::fputs(line.c_str(), f);
    }
    std::fclose(f);
    return SMCGPU_OK;
}

extern "C" int32_t smcgpu_write_point_cloud(smcgpu_ctx *ctx, const char *prefix, int32_t n, int32_t nr,
                                           const double *points) {
    if (!ctx) return SMCGPU_ERR_ARG;
    if (!prefix || n < 0 || nr < 1 || (n > 0 && !points))
        return ctx->fail(SMCGPU_ERR_ARG, "write_point_cloud: bad arguments");
    // point_cloud's files (main.f90:785-805): one file per plane, named
    // prefix//iplane with iplane written as I1; records of x, y, z, uxi,
    // ueta, |u| in f12.5, geometry by geometry, patch by patch
    const smc::MeshPattern &m = ctx->mesh;
    const size_t per = (size_t)m.npatch * nr * nr;
    std::string line;
    for (int ip = 0; ip < m.nplane; ++ip) {
        std::string name = std::string(prefix) + (ip + 1 < 10 ? std::string(1, (char)('1' + ip)) : std::string("*"));
        FILE *f = std::fopen(name.c_str(), "w");
        if (!f) return ctx->fail(SMCGPU_ERR_ARG, "write_point_cloud: cannot open " + name);
        for (int t = 0; t < n; ++t)
            for (size_t q = (size_t)m.patch_off[ip] * nr * nr; q < (size_t)m.patch_off[ip + 1] * nr * nr; ++q) {
                const double *pt = points + ((size_t)t * per + q) * 6;
                line.clear();
                for (int k = 0; k < 6; ++k) line += smc::fortran_f(pt[k], 12, 5);
                line += '\n';
                std::fputs(line.c_str(), f);
            }
        std::fclose(f);
    }
    return SMCGPU_OK;
}
