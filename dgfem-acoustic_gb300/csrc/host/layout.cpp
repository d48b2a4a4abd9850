// Element-centric device layout (see layout.h) and its C ABI for inspection.
#include "layout.h"

#include <algorithm>
#include <cmath>
#include <exception>

#include "capi_common.h"
#include "refel.h"

namespace dg {

namespace {

// Curved elements: those whose Jacobian differs between the points of the
// element rule by more than 1e-11 of its largest entry.
std::vector<int> curved_elements(const dg_mesh_desc &m, int dim) {
    std::vector<int> out;
    const int ng = m.el_num_int_pts;
    if (ng <= 0 || !m.el_jacobians_qp) return out;
    for (int e = 0; e < m.num_el; ++e) {
        const double *J0 = &m.el_jacobians_qp[(size_t)e * ng * 9];
        double scale = 0, dev = 0;
        for (int u = 0; u < dim; ++u)
            for (int x = 0; x < 3; ++x) scale = std::max(scale, std::fabs(J0[u * 3 + x]));
        for (int g = 1; g < ng; ++g) {
            const double *J = J0 + (size_t)g * 9;
            for (int u = 0; u < dim; ++u)
                for (int x = 0; x < 3; ++x) dev = std::max(dev, std::fabs(J[u * 3 + x] - J0[u * 3 + x]));
        }
        if (dev > 1e-11 * scale) out.push_back(e);
    }
    return out;
}

// Per-point data of the curved elements (Mesh.cpp:440-466 mass, 476-489
// stiffness, 500-557 surface integral and scatter, 569-674 boundary traces).
std::string build_curved(const dg_mesh_desc &m, int flux_sign, const RefElement &re, Layout &L,
                         const std::vector<int> &cel) {
    CurvedLayout &Cv = L.curved;
    const int dim = L.dim, np = L.np, nf = L.nf, nfp = L.nfp, K = L.K;
    const int ng = m.el_num_int_pts, ngf = m.f_num_int_pts;
    if (!m.el_int_param_coords || !m.el_basis_fcts || !m.el_ugrad_basis_fcts || !m.el_jacobian_dets_qp)
        return "curved elements need the per-point element arrays";
    if (ngf <= 0 || !m.f_int_param_coords || !m.f_basis_fcts || !m.f_normals_qp || !m.f_jacobian_dets_qp)
        return "curved elements need the per-point face arrays";
    const int C = (int)cel.size();
    Cv.C = C; Cv.ng = ng; Cv.ngf = ngf;
    Cv.el = cel;
    Cv.slot.assign(K, -1);
    for (int c = 0; c < C; ++c) Cv.slot[cel[c]] = c;
    Cv.phi.assign(m.el_basis_fcts, m.el_basis_fcts + (size_t)ng * np);
    Cv.dphi.assign((size_t)dim * ng * np, 0.0);
    for (int u = 0; u < dim; ++u)
        for (int g = 0; g < ng; ++g)
            for (int i = 0; i < np; ++i)
                Cv.dphi[((size_t)u * ng + g) * np + i] = m.el_ugrad_basis_fcts[((size_t)g * np + i) * 3 + u];
    Cv.fphi.assign(m.f_basis_fcts, m.f_basis_fcts + (size_t)ngf * nfp);
    Cv.minv.assign((size_t)C * np * np, 0.0);
    Cv.wm.assign((size_t)C * ng * dim * dim, 0.0);
    Cv.wdet.assign((size_t)C * ng, 0.0);
    Cv.fw.assign((size_t)C * nf * ngf * 4, 0.0);
    Cv.fconn.assign((size_t)C * nf * 2, -1);
    Cv.fmap.assign((size_t)C * nf * 2 * nfp, 0);
    std::vector<double> M((size_t)np * np), A(dim * dim);
    for (int c = 0; c < C; ++c) {
        const int e = cel[c];
        const double *detj = &m.el_jacobian_dets_qp[(size_t)e * ng];
        // mass matrix summed over the points in the reference's order, then
        // inverted (Mesh.cpp:454-465)
        for (int i = 0; i < np; ++i)
            for (int j = 0; j < np; ++j) {
                double s = 0;
                for (int g = 0; g < ng; ++g)
                    s += m.el_basis_fcts[g * np + i] * m.el_basis_fcts[g * np + j] * m.el_int_param_coords[g * 4 + 3] *
                         detj[g];
                M[(size_t)i * np + j] = s;
            }
        if (!lu_inverse(M, np)) return "singular mass matrix of curved element " + std::to_string(e);
        std::copy(M.begin(), M.end(), Cv.minv.begin() + (size_t)c * np * np);
        for (int g = 0; g < ng; ++g) {
            if (!(detj[g] > 0)) return "non-positive Jacobian determinant in curved element " + std::to_string(e);
            const double *J = &m.el_jacobians_qp[((size_t)e * ng + g) * 9];
            for (int u = 0; u < dim; ++u)
                for (int x = 0; x < dim; ++x) A[u * dim + x] = J[u * 3 + x];
            if (!lu_inverse(A, dim)) return "singular Jacobian in curved element " + std::to_string(e);
            const double wd = m.el_int_param_coords[g * 4 + 3] * detj[g];
            Cv.wdet[(size_t)c * ng + g] = wd;
            for (int k = 0; k < dim * dim; ++k) Cv.wm[((size_t)c * ng + g) * dim * dim + k] = wd * A[k];
        }
        for (int lf = 0; lf < nf; ++lf) {
            const int f = m.el_f_ids[(size_t)e * nf + lf];
            const int side = (m.f_nbr_el_ids[f * 2] == e) ? 0 : 1;
            const int o = m.el_f_orientation[(size_t)e * nf + lf];
            for (int g = 0; g < ngf; ++g) {
                double *w = &Cv.fw[(((size_t)c * nf + lf) * ngf + g) * 4];
                for (int x = 0; x < dim; ++x) w[x] = o * m.f_normals_qp[((size_t)f * ngf + g) * 3 + x];
                w[3] = m.f_int_param_coords[g * 4 + 3] * m.f_jacobian_dets_qp[(size_t)f * ngf + g];
            }
            int *cn = &Cv.fconn[((size_t)c * nf + lf) * 2];
            uint8_t *own = &Cv.fmap[(((size_t)c * nf + lf) * 2) * nfp];
            uint8_t *nbm = own + nfp;
            for (int k = 0; k < nfp; ++k) {
                const int v = m.f_n_to_el_n_ids[((size_t)f * nfp + k) * 2 + side];
                if (v < 0 || v >= np) return "face node map out of range";
                own[k] = (uint8_t)v;
            }
            if (m.f_is_boundary[f]) {
                cn[0] = -1;
                cn[1] = (m.f_bc[f] == 1 ? 1 : 2) << 5;
                continue;
            }
            const int nb = m.f_nbr_el_ids[f * 2 + 1 - side];
            for (int k = 0; k < nfp; ++k) {
                const int v = m.f_n_to_el_n_ids[((size_t)f * nfp + k) * 2 + 1 - side];
                if (v < 0 || v >= np) return "face node map out of range";
                nbm[k] = (uint8_t)v;
            }
            int tau = (side == 0) ? m.fc * o : -m.fc * o;
            if (flux_sign == DG_FLUX_UPWIND) tau = 1;
            cn[0] = nb;
            cn[1] = tau < 0 ? 128 : 0;
        }
    }
    for (int e = 0; e < K; ++e)
        if (Cv.slot[e] < 0) Cv.affine.push_back(e);
    (void)re;
    return "";
}

}  // namespace

// connectivity word (see stage_kernel.cuh): bits 0-1 neighbour's local face,
// 2-4 permutation, 5-6 kind (0 interior, 1 reflecting, 2 absorbing), 7 tau<0
std::string build_layout(const dg_mesh_desc &m, int flux_sign, Layout &L) {
    if (m.dim != 2 && m.dim != 3) return "dimension must be 2 or 3";
    if (m.order < 1 || m.order > 5) return "order must be in 1..5";
    RefElement re = make_refel(m.dim, m.order);
    const int dim = m.dim, np = re.np, nf = re.nf, nfp = re.nfp, K = m.num_el, F = m.f_num;
    if (m.el_num_nodes != np || m.f_num_per_el != nf || m.f_num_nodes != nfp)
        return "element/face node counts do not match the element order";
    if (K < 1 || F < 1) return "empty mesh";
    if (!m.el_jacobians || !m.el_jacobian_dets || !m.f_normals || !m.f_jacobian_dets || !m.el_f_ids ||
        !m.el_f_orientation || !m.f_nbr_el_ids || !m.f_n_to_el_n_ids || !m.f_bc || !m.f_is_boundary)
        return "null mesh array";
    L = Layout();
    L.dim = dim; L.order = m.order; L.np = np; L.nf = nf; L.nfp = nfp; L.nq = dim + 1; L.nperm = re.nperm; L.K = K;
    L.geo.assign((size_t)K * dim * dim, 0.0);
    L.fgeo.assign((size_t)K * nf * 4, 0.0);
    L.conn.assign((size_t)K * nf * 2, 0);
    L.detj.assign(m.el_jacobian_dets, m.el_jacobian_dets + K);
    std::vector<int> target(nfp);
    for (int e = 0; e < K; ++e) {
        std::vector<double> A(dim * dim);
        for (int u = 0; u < dim; ++u)
            for (int x = 0; x < dim; ++x) A[u * dim + x] = m.el_jacobians[(size_t)e * 9 + u * 3 + x];
        if (!lu_inverse(A, dim)) return "singular element Jacobian";
        for (int k = 0; k < dim * dim; ++k) L.geo[(size_t)e * dim * dim + k] = A[k];
        double dje = m.el_jacobian_dets[e];
        if (!(dje != 0)) return "zero element Jacobian determinant";
        for (int lf = 0; lf < nf; ++lf) {
            int f = m.el_f_ids[(size_t)e * nf + lf];
            if (f < 0 || f >= F) return "face id out of range";
            int side;
            if (m.f_nbr_el_ids[f * 2] == e) side = 0;
            else if (m.f_nbr_el_ids[f * 2 + 1] == e) side = 1;
            else return "element is not a neighbour of its own face";
            int o = m.el_f_orientation[(size_t)e * nf + lf];
            double *g = &L.fgeo[((size_t)e * nf + lf) * 4];
            for (int x = 0; x < dim; ++x) g[x] = o * m.f_normals[(size_t)f * 3 + x];
            g[dim] = m.f_jacobian_dets[f] / dje;
            int *cn = &L.conn[((size_t)e * nf + lf) * 2];
            if (m.f_is_boundary[f]) {
                cn[0] = -1;
                cn[1] = (m.f_bc[f] == 1 ? 1 : 2) << 5;
                continue;
            }
            int nb = m.f_nbr_el_ids[f * 2 + 1 - side];
            if (nb < 0 || nb >= K) return "interior face without a second neighbour";
            int nlf = -1;
            for (int l = 0; l < nf; ++l)
                if (m.el_f_ids[(size_t)nb * nf + l] == f) nlf = l;
            if (nlf < 0) return "neighbour does not list the face";
            for (int kl = 0; kl < nfp; ++kl) {
                int vi = re.fmask[lf * nfp + kl];
                int k = -1;
                for (int kk = 0; kk < nfp; ++kk)
                    if (m.f_n_to_el_n_ids[((size_t)f * nfp + kk) * 2 + side] == vi) k = kk;
                if (k < 0) return "face node map does not match the element's face";
                int nvi = m.f_n_to_el_n_ids[((size_t)f * nfp + k) * 2 + 1 - side];
                int kn = -1;
                for (int kk = 0; kk < nfp; ++kk)
                    if (re.fmask[nlf * nfp + kk] == nvi) kn = kk;
                if (kn < 0) return "face node map does not match the neighbour's face";
                target[kl] = kn;
            }
            int pm = -1;
            for (int p = 0; p < re.nperm && pm < 0; ++p) {
                bool ok = true;
                for (int kl = 0; kl < nfp && ok; ++kl) ok = re.perm[p * nfp + kl] == target[kl];
                if (ok) pm = p;
            }
            if (pm < 0) return "non-conforming face (no face symmetry matches)";
            // jump sign seen from this element (Mesh.cpp:524 scattered with
            // the orientation at Mesh.cpp:554): fc*o on the first neighbour's
            // side, -fc*o on the second's
            int tau = (side == 0) ? m.fc * o : -m.fc * o;
            if (flux_sign == DG_FLUX_UPWIND) tau = 1;
            cn[0] = nb;
            cn[1] = nlf | (pm << 2) | (tau < 0 ? 128 : 0);
        }
    }
    // operators: D as [u][j][i] (transpose of D_u[i][j]), then LIFT [lf*nfp+k][i]
    L.ops.assign((size_t)dim * np * np, 0.0);
    for (int u = 0; u < dim; ++u)
        for (int i = 0; i < np; ++i)
            for (int j = 0; j < np; ++j) L.ops[((size_t)u * np + j) * np + i] = re.D[((size_t)u * np + i) * np + j];
    for (int lf = 0; lf < nf; ++lf)
        for (int k = 0; k < nfp; ++k)
            for (int i = 0; i < np; ++i) L.ops.push_back(re.lift[((size_t)lf * np + i) * nfp + k]);
    for (int v : re.fmask) L.tabs.push_back((uint8_t)v);
    for (int v : re.perm) L.tabs.push_back((uint8_t)v);
    L.mass = re.mass;
    std::vector<int> cel = curved_elements(m, dim);
    if (!cel.empty()) return build_curved(m, flux_sign, re, L, cel);
    return "";
}

}  // namespace dg

struct dg_layout {
    dg::Layout L;
};

extern "C" {

int dg_layout_build(const dg_mesh_desc *m, int flux_sign, dg_layout **out) {
    if (!m || !out) return dg::fail(DG_ERR_ARG, "null argument");
    auto *h = new dg_layout();
    std::string err;
    try {
        err = dg::build_layout(*m, flux_sign, h->L);
    } catch (std::exception &e) {
        err = e.what();
    }
    if (!err.empty()) {
        delete h;
        return dg::fail(DG_ERR_MESH, err);
    }
    if (h->L.curved.C > 0) {
        delete h;
        return dg::fail(DG_ERR_UNSUPPORTED, "the element-centric layout view holds straight-sided elements only; "
                                            "meshes with curved elements run through dg_create");
    }
    *out = h;
    return DG_OK;
}

int dg_layout_get(const dg_layout *h, dg_layout_view *v) {
    if (!h || !v) return dg::fail(DG_ERR_ARG, "null argument");
    const dg::Layout &L = h->L;
    v->dim = L.dim; v->order = L.order; v->np = L.np; v->nf = L.nf; v->nfp = L.nfp; v->nq = L.nq;
    v->nperm = L.nperm; v->num_el = L.K;
    v->geo = L.geo.data(); v->fgeo = L.fgeo.data(); v->conn = L.conn.data(); v->ops = L.ops.data();
    v->n_ops = (int)L.ops.size(); v->tabs = L.tabs.data(); v->n_tabs = (int)L.tabs.size();
    v->mass = L.mass.data();
    return DG_OK;
}

void dg_layout_free(dg_layout *h) { delete h; }

}  // extern "C"
