// C ABI of the host mesh layer (include/dgmesh.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../../include/dgmesh.h"
#include "capi_common.h"
#include "config.h"
#include "mesh_io.h"
#include "precompute.h"

namespace dg {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
}  // namespace dg

using namespace dg;

struct dgm_mesh {
    RawMesh m;
    // flattened views
    std::vector<int> phys_dim, phys_tag, phys_off, phys_nodes;
    std::vector<const char *> phys_name;
    void flatten() {
        phys_dim.clear(); phys_tag.clear(); phys_off.assign(1, 0); phys_nodes.clear(); phys_name.clear();
        for (auto &g : m.phys) {
            phys_dim.push_back(g.dim);
            phys_tag.push_back(g.tag);
            phys_name.push_back(g.name.c_str());
            phys_nodes.insert(phys_nodes.end(), g.nodes.begin(), g.nodes.end());
            phys_off.push_back((int)phys_nodes.size());
        }
    }
};

struct dgm_precomp {
    Precomp p;
};

struct dgm_config {
    Config c;
    std::vector<double> src, ic;
    std::vector<int> bc_tag, bc_refl;
};

extern "C" {

const char *dg_last_error(void) { return g_last_error.c_str(); }

int dgm_read_msh(const char *path, dgm_mesh **out) {
    if (!path || !out) return fail(DG_ERR_ARG, "null argument");
    return guarded([&]() {
        std::unique_ptr<dgm_mesh> h(new dgm_mesh());
        std::string err = read_msh(path, h->m);
        if (!err.empty()) return fail(DG_ERR_IO, err);
        h->flatten();
        *out = h.release();
        return DG_OK;
    });
}

int dgm_write_msh(const dgm_mesh *m, const char *path) {
    if (!m || !path) return fail(DG_ERR_ARG, "null argument");
    std::string err = write_msh(m->m, path);
    return err.empty() ? DG_OK : fail(DG_ERR_IO, err);
}

static std::vector<std::string> names(const char *const *n, int cnt) {
    std::vector<std::string> v(cnt);
    for (int i = 0; i < cnt; ++i) v[i] = (n && n[i]) ? n[i] : "";
    return v;
}

int dgm_box_tri(int nx, int ny, const double lo[2], const double hi[2], int order, const char *const side_names[4],
                dgm_mesh **out) {
    if (!lo || !hi || !out) return fail(DG_ERR_ARG, "null argument");
    return guarded([&]() {
        std::unique_ptr<dgm_mesh> h(new dgm_mesh());
        std::string err = box_tri(nx, ny, lo, hi, order, names(side_names, 4), h->m);
        if (!err.empty()) return fail(DG_ERR_ARG, err);
        h->flatten();
        *out = h.release();
        return DG_OK;
    });
}

int dgm_box_tet(int nx, int ny, int nz, const double lo[3], const double hi[3], int order,
                const char *const side_names[6], const int *removed, int nremoved, const char *obstacle_name,
                dgm_mesh **out) {
    if (!lo || !hi || !out) return fail(DG_ERR_ARG, "null argument");
    if (removed && nremoved < 0) return fail(DG_ERR_ARG, "negative count of removed cells");
    return guarded([&]() {
        std::unique_ptr<dgm_mesh> h(new dgm_mesh());
        std::vector<int> rem(removed, removed + (removed ? nremoved : 0));
        std::string err = box_tet(nx, ny, nz, lo, hi, order, names(side_names, 6), rem,
                                  obstacle_name ? obstacle_name : "", h->m);
        if (!err.empty()) return fail(DG_ERR_ARG, err);
        h->flatten();
        *out = h.release();
        return DG_OK;
    });
}

int dgm_get_raw(const dgm_mesh *h, dgm_raw *o) {
    if (!h || !o) return fail(DG_ERR_ARG, "null argument");
    const RawMesh &m = h->m;
    o->dim = m.dim; o->order = m.order; o->el_type = m.el_type; o->np = m.np;
    o->num_nodes = (int)m.node_tags.size(); o->node_tags = m.node_tags.data(); o->xyz = m.xyz.data();
    o->num_el = m.num_el(); o->el_tags = m.el_tags.data(); o->el_nodes = m.el_nodes.data();
    o->num_phys = (int)m.phys.size();
    o->phys_dim = h->phys_dim.data(); o->phys_tag = h->phys_tag.data();
    o->phys_name = h->phys_name.data();
    o->phys_node_offsets = h->phys_off.data(); o->phys_nodes = h->phys_nodes.data();
    return DG_OK;
}

int dgm_set_nodes(dgm_mesh *h, const double *xyz) {
    if (!h || !xyz) return fail(DG_ERR_ARG, "null argument");
    for (size_t i = 0; i < h->m.xyz.size(); ++i)
        if (!std::isfinite(xyz[i])) return fail(DG_ERR_ARG, "non-finite node coordinate");
    std::copy(xyz, xyz + h->m.xyz.size(), h->m.xyz.begin());
    return DG_OK;
}

void dgm_free_mesh(dgm_mesh *m) { delete m; }

int dgm_precompute(const dgm_mesh *m, int nbc, const int *tags, const int *refl, dgm_precomp **out) {
    if (!m || !out || (nbc > 0 && (!tags || !refl))) return fail(DG_ERR_ARG, "null argument");
    std::vector<std::pair<int, bool>> bcs;
    for (int i = 0; i < nbc; ++i) bcs.push_back({tags[i], refl[i] != 0});
    auto *h = new dgm_precomp();
    std::string err;
    try {
        err = precompute(m->m, bcs, h->p);
    } catch (std::exception &e) {
        err = e.what();
    }
    if (!err.empty()) { delete h; return fail(DG_ERR_MESH, err); }
    *out = h;
    return DG_OK;
}

int dgm_get_desc(const dgm_precomp *h, dg_mesh_desc *d) {
    if (!h || !d) return fail(DG_ERR_ARG, "null argument");
    fill_desc(h->p, *d);
    return DG_OK;
}

int dgm_get_curved(const dgm_precomp *h, int *ncurved, const unsigned char **flags) {
    if (!h || !ncurved) return fail(DG_ERR_ARG, "null argument");
    *ncurved = h->p.ncurved;
    if (flags) *flags = h->p.el_curved.data();
    return DG_OK;
}

int dgm_get_dof_coords(const dgm_precomp *h, const double **xyz) {
    if (!h || !xyz) return fail(DG_ERR_ARG, "null argument");
    *xyz = h->p.dof_xyz.data();
    return DG_OK;
}

int dgm_get_face_node_tags(const dgm_precomp *h, const int **tags) {
    if (!h || !tags) return fail(DG_ERR_ARG, "null argument");
    *tags = h->p.f_node_tags.data();
    return DG_OK;
}

double dgm_min_edge(const dgm_precomp *h) {
    if (!h) return 0;
    const Precomp &p = h->p;
    double best = std::numeric_limits<double>::infinity();
    int nv = p.dim + 1;
    for (int e = 0; e < p.K; ++e)
        for (int a = 0; a < nv; ++a)
            for (int b = a + 1; b < nv; ++b) {
                const double *xa = &p.dof_xyz[((size_t)e * p.np + a) * 3];
                const double *xb = &p.dof_xyz[((size_t)e * p.np + b) * 3];
                double d = std::sqrt((xa[0] - xb[0]) * (xa[0] - xb[0]) + (xa[1] - xb[1]) * (xa[1] - xb[1]) +
                                     (xa[2] - xb[2]) * (xa[2] - xb[2]));
                best = std::min(best, d);
            }
    return best;
}

void dgm_free_precomp(dgm_precomp *p) { delete p; }

int dgm_gaussian_ic(const dgm_precomp *h, double x, double y, double z, double size, double amp, double *u0) {
    if (!h || !u0) return fail(DG_ERR_ARG, "null argument");
    const Precomp &p = h->p;
    size_t n = (size_t)p.K * p.np;
    for (size_t i = 0; i < n; ++i) {
        const double *c = &p.dof_xyz[i * 3];
        u0[i] += amp * std::exp(-((c[0] - x) * (c[0] - x) + (c[1] - y) * (c[1] - y) + (c[2] - z) * (c[2] - z)) / size);
    }
    return DG_OK;
}

int dgm_source_dofs(const dgm_precomp *h, double x, double y, double z, double size, int *idx, int cap, int *count) {
    if (!h || !count) return fail(DG_ERR_ARG, "null argument");
    const Precomp &p = h->p;
    size_t n = (size_t)p.K * p.np;
    int c = 0;
    for (size_t i = 0; i < n; ++i) {
        const double *q = &p.dof_xyz[i * 3];
        if (std::pow(q[0] - x, 2) + std::pow(q[1] - y, 2) + std::pow(q[2] - z, 2) < std::pow(size, 2)) {
            if (idx && c < cap) idx[c] = (int)i;
            ++c;
        }
    }
    *count = c;
    return DG_OK;
}

int dgm_parse_config(const char *path, const dgm_mesh *m, dgm_config **out) {
    if (!path || !m || !out) return fail(DG_ERR_ARG, "null argument");
    return guarded([&]() {
        std::unique_ptr<dgm_config> h(new dgm_config());
        std::string err = parse_config(path, m->m, h->c);
        if (!err.empty()) return fail(DG_ERR_CONFIG, err);
        for (auto &s : h->c.sources) h->src.insert(h->src.end(), s.begin(), s.end());
        for (auto &s : h->c.initConditions) h->ic.insert(h->ic.end(), s.begin(), s.end());
        for (auto &kv : h->c.physBCs) { h->bc_tag.push_back(kv.first); h->bc_refl.push_back(kv.second ? 1 : 0); }
        *out = h.release();
        return DG_OK;
    });
}

int dgm_get_config(const dgm_config *h, dgm_config_view *v) {
    if (!h || !v) return fail(DG_ERR_ARG, "null argument");
    const Config &c = h->c;
    v->time_start = c.timeStart; v->time_end = c.timeEnd; v->time_step = c.timeStep; v->time_rate = c.timeRate;
    v->num_threads = c.numThreads;
    for (int k = 0; k < 3; ++k) v->v0[k] = c.v0[k];
    v->rho0 = c.rho0; v->c0 = c.c0;
    v->num_sources = (int)c.sources.size(); v->sources = h->src.data();
    v->num_ics = (int)c.initConditions.size(); v->ics = h->ic.data();
    v->num_bcs = (int)h->bc_tag.size(); v->bc_phys_tags = h->bc_tag.data(); v->bc_reflecting = h->bc_refl.data();
    v->element_type = c.elementType.c_str(); v->time_int_method = c.timeIntMethod.c_str();
    v->save_file = c.saveFile.c_str(); v->precision = c.precision.c_str(); v->flux_sign = c.fluxSign.c_str();
    return DG_OK;
}

void dgm_free_config(dgm_config *c) { delete c; }

}  // extern "C"
