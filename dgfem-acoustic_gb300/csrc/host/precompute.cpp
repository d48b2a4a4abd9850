// Reference-semantics mesh precompute (affine and curved simplices).
#include "precompute.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <unordered_map>

#include "rules.h"

namespace dg {

namespace {

void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
double norm3(const double *a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// gmsh's completion of the Jacobian rows of a lower-dimensional element:
// 1D: b = (a1,-a0,0) when the tangent is dominant in x or y, else (0,a2,-a1);
//     c = a x b, both normalised.  2D: c = normalised (row0 x row1).
void complete_jacobian(int edim, double jac[3][3]) {
    if (edim == 1) {
        const double *a = jac[0];
        double b[3], c[3];
        if ((std::fabs(a[0]) >= std::fabs(a[1]) && std::fabs(a[0]) >= std::fabs(a[2])) ||
            (std::fabs(a[1]) >= std::fabs(a[0]) && std::fabs(a[1]) >= std::fabs(a[2]))) {
            b[0] = a[1]; b[1] = -a[0]; b[2] = 0.0;
        } else {
            b[0] = 0.0; b[1] = a[2]; b[2] = -a[1];
        }
        double nb = norm3(b);
        for (int k = 0; k < 3; ++k) b[k] /= nb;
        cross3(a, b, c);
        double nc = norm3(c);
        for (int k = 0; k < 3; ++k) c[k] /= nc;
        for (int k = 0; k < 3; ++k) { jac[1][k] = b[k]; jac[2][k] = c[k]; }
    } else if (edim == 2) {
        double c[3];
        cross3(jac[0], jac[1], c);
        double nc = norm3(c);
        for (int k = 0; k < 3; ++k) jac[2][k] = c[k] / nc;
    }
}

struct VecHash {
    size_t operator()(const std::vector<int> &v) const {
        size_t h = 1469598103934665603ull;
        for (int x : v) { h ^= (size_t)(unsigned)x; h *= 1099511628211ull; }
        return h;
    }
};

// Per-point element data (Mesh.cpp:31-38 and the gradient solve at 58-71):
// at every point g of the Gauss(2p) rule, J = sum_k x_k dphi_k/du (gmsh
// storage [u*3+x], completed for 2D elements) and its determinant.  The
// first-point arrays are replaced by the values at point 0.
template <typename NodeFn>
std::string element_points(const RawMesh &m, const RefElement &re, NodeFn X, Precomp &P) {
    const int dim = P.dim, np = P.np, K = P.K;
    QuadRule r = quad_rule(dim, 2 * P.order);
    if (r.n == 0) return "no element quadrature rule for this order";
    const int ng = r.n;
    P.ng = ng;
    P.el_qp = r.uvwq;
    P.el_phi.assign((size_t)ng * np, 0.0);
    P.el_dphi.assign((size_t)ng * np * 3, 0.0);
    for (int g = 0; g < ng; ++g)
        lagrange_eval(dim, P.order, &r.uvwq[g * 4], &P.el_phi[(size_t)g * np], &P.el_dphi[(size_t)g * np * 3]);
    P.el_jac_qp.assign((size_t)K * ng * 9, 0.0);
    P.el_detj_qp.assign((size_t)K * ng, 0.0);
    for (int e = 0; e < K; ++e) {
        const int *en = &m.el_nodes[(size_t)e * np];
        for (int g = 0; g < ng; ++g) {
            double jac[3][3] = {};
            for (int k = 0; k < np; ++k) {
                const double *xk = X(en[k]);
                const double *dk = &P.el_dphi[((size_t)g * np + k) * 3];
                for (int u = 0; u < dim; ++u)
                    for (int x = 0; x < 3; ++x) jac[u][x] += xk[x] * dk[u];
            }
            double det;
            if (dim == 2) {
                double c[3];
                cross3(jac[0], jac[1], c);
                det = norm3(c);
                complete_jacobian(2, jac);
            } else {
                double c[3];
                cross3(jac[1], jac[2], c);
                det = jac[0][0] * c[0] + jac[0][1] * c[1] + jac[0][2] * c[2];
            }
            if (!(det > 0)) return "inverted or degenerate curved element " + std::to_string(e);
            double *J = &P.el_jac_qp[((size_t)e * ng + g) * 9];
            for (int u = 0; u < 3; ++u)
                for (int x = 0; x < 3; ++x) J[u * 3 + x] = jac[u][x];
            P.el_detj_qp[(size_t)e * ng + g] = det;
        }
        for (int k = 0; k < 9; ++k) P.el_jac[(size_t)e * 9 + k] = P.el_jac_qp[(size_t)e * ng * 9 + k];
        P.el_detj[e] = P.el_detj_qp[(size_t)e * ng];
    }
    (void)re;
    return "";
}

// Per-point face data (Mesh.cpp:135-194): face Jacobian from all face nodes
// (completed), determinant, gradients of face basis functions 0 and 1 by the
// transposed-Jacobian solve, normal = grad0 x grad1 (3D) or grad0 x (0,0,-1)
// (2D), sign aligned with point 0 as the reference does (3D: the normal at
// point 0; 2D: grad0 at point 0), normalised.  The first-point face arrays
// are replaced by the values at point 0.
template <typename NodeFn>
std::string face_points(const RefElement &re, NodeFn X, Precomp &P) {
    const int dim = P.dim, nfp = P.nfp, F = P.F, fdim = dim - 1;
    QuadRule r = quad_rule(fdim, 2 * P.order);
    if (r.n == 0) return "no face quadrature rule for this order";
    const int ngf = r.n;
    P.ngf = ngf;
    P.f_qp = r.uvwq;
    P.f_phi.assign((size_t)ngf * nfp, 0.0);
    std::vector<double> fd((size_t)ngf * nfp * 3, 0.0);
    for (int g = 0; g < ngf; ++g)
        lagrange_eval(fdim, P.order, &r.uvwq[g * 4], &P.f_phi[(size_t)g * nfp], &fd[(size_t)g * nfp * 3]);
    P.f_normal_qp.assign((size_t)F * ngf * 3, 0.0);
    P.f_detj_qp.assign((size_t)F * ngf, 0.0);
    for (int f = 0; f < F; ++f) {
        const int *fn = &P.f_node_tags[(size_t)f * nfp];
        double grad0_first[3] = {0, 0, 0};
        for (int g = 0; g < ngf; ++g) {
            double jac[3][3] = {};
            for (int k = 0; k < nfp; ++k) {
                const double *xk = X(fn[k]);
                const double *dk = &fd[((size_t)g * nfp + k) * 3];
                for (int u = 0; u < fdim; ++u)
                    for (int x = 0; x < 3; ++x) jac[u][x] += xk[x] * dk[u];
            }
            double det;
            if (fdim == 1) {
                det = norm3(jac[0]);
            } else {
                double c[3];
                cross3(jac[0], jac[1], c);
                det = norm3(c);
            }
            complete_jacobian(fdim, jac);
            double A[9];
            for (int rr = 0; rr < dim; ++rr)
                for (int cc = 0; cc < dim; ++cc) A[rr * dim + cc] = jac[rr][cc];
            const double *d0 = &fd[((size_t)g * nfp + 0) * 3];
            const double *d1 = &fd[((size_t)g * nfp + 1) * 3];
            double g0[3] = {d0[0], fdim == 2 ? d0[1] : 0.0, 0.0};
            double g1[3] = {d1[0], fdim == 2 ? d1[1] : 0.0, 0.0};
            if (!lu_solve(A, g0, dim) || !lu_solve(A, g1, dim)) return "singular face Jacobian";
            double n[3];
            double *nq = &P.f_normal_qp[((size_t)f * ngf + g) * 3];
            if (dim == 2) {
                double z[3] = {0, 0, -1};
                cross3(g0, z, n);
                if (g == 0)
                    for (int x = 0; x < 3; ++x) grad0_first[x] = g0[x];
                if (g0[0] * grad0_first[0] + g0[1] * grad0_first[1] + g0[2] * grad0_first[2] < 0)
                    for (int x = 0; x < 3; ++x) n[x] = -n[x];
            } else {
                cross3(g0, g1, n);
                const double *n0 = &P.f_normal_qp[(size_t)f * ngf * 3];
                if (g != 0 && n0[0] * n[0] + n0[1] * n[1] + n0[2] * n[2] < 0)
                    for (int x = 0; x < 3; ++x) n[x] = -n[x];
            }
            double nn = norm3(n);
            if (!(nn > 0)) return "degenerate face normal at a quadrature point of face " + std::to_string(f);
            for (int x = 0; x < 3; ++x) nq[x] = n[x] / nn;
            P.f_detj_qp[(size_t)f * ngf + g] = det;
        }
        for (int x = 0; x < 3; ++x) P.f_normal[(size_t)f * 3 + x] = P.f_normal_qp[(size_t)f * ngf * 3 + x];
        P.f_detj[f] = P.f_detj_qp[(size_t)f * ngf];
    }
    (void)re;
    return "";
}

}  // namespace

void fill_desc(const Precomp &p, dg_mesh_desc &d) {
    d = dg_mesh_desc();
    d.dim = p.dim; d.order = p.order; d.num_el = p.K; d.el_num_nodes = p.np;
    d.f_num = p.F; d.f_num_per_el = p.nf; d.f_num_nodes = p.nfp; d.fc = p.fc;
    d.el_jacobians = p.el_jac.data(); d.el_jacobian_dets = p.el_detj.data();
    d.f_normals = p.f_normal.data(); d.f_jacobian_dets = p.f_detj.data();
    d.el_f_ids = p.el_f_ids.data(); d.el_f_orientation = p.el_f_orient.data();
    d.f_nbr_el_ids = p.f_nbr.data(); d.f_n_to_el_n_ids = p.f_n_to_el_n.data();
    d.f_bc = p.f_bc.data(); d.f_is_boundary = p.f_is_bnd.data();
    if (p.ncurved > 0) {
        d.el_num_int_pts = p.ng;
        d.el_int_param_coords = p.el_qp.data();
        d.el_basis_fcts = p.el_phi.data();
        d.el_ugrad_basis_fcts = p.el_dphi.data();
        d.el_jacobians_qp = p.el_jac_qp.data();
        d.el_jacobian_dets_qp = p.el_detj_qp.data();
        d.f_num_int_pts = p.ngf;
        d.f_int_param_coords = p.f_qp.data();
        d.f_basis_fcts = p.f_phi.data();
        d.f_normals_qp = p.f_normal_qp.data();
        d.f_jacobian_dets_qp = p.f_detj_qp.data();
    }
}

std::string precompute(const RawMesh &m, const std::vector<std::pair<int, bool>> &physical_bcs, Precomp &P) {
    P = Precomp();
    if (m.dim != 2 && m.dim != 3) return "only 2D and 3D meshes are supported";
    RefElement re = make_refel(m.dim, m.order);
    const int dim = m.dim, np = re.np, nf = re.nf, nfp = re.nfp;
    const int K = m.num_el();
    if (np != m.np) return "element node count mismatch";
    P.dim = dim; P.order = m.order; P.K = K; P.np = np; P.nf = nf; P.nfp = nfp;
    P.fc = (dim == 3 && m.order != 1) ? -1 : 1;
    P.el_node_tags = m.el_nodes;

    // node tag -> coordinates: a dense table, or a hash map when the tags
    // are sparse (tags are positive and unique)
    if (m.xyz.size() != m.node_tags.size() * 3) return "node coordinate count mismatch";
    int maxtag = 0;
    for (int t : m.node_tags) {
        if (t < 1) return "invalid node tag " + std::to_string(t);
        maxtag = std::max(maxtag, t);
    }
    const bool dense = (size_t)maxtag <= 8 * m.node_tags.size() + 1024;
    std::vector<int> idx(dense ? (size_t)maxtag + 1 : 0, -1);
    std::unordered_map<int, int> sparse;
    for (size_t i = 0; i < m.node_tags.size(); ++i) {
        const int t = m.node_tags[i];
        const bool fresh = dense ? idx[t] < 0 : sparse.find(t) == sparse.end();
        if (!fresh) return "duplicate node tag " + std::to_string(t);
        if (dense) idx[t] = (int)i;
        else sparse[t] = (int)i;
    }
    auto X = [&](int tag) -> const double * {
        if (tag < 1 || tag > maxtag) return nullptr;
        int i = -1;
        if (dense) {
            i = idx[tag];
        } else {
            auto it = sparse.find(tag);
            if (it != sparse.end()) i = it->second;
        }
        return i < 0 ? nullptr : &m.xyz[(size_t)i * 3];
    };
    for (int t : m.el_nodes)
        if (!X(t)) return "element references an unknown node tag " + std::to_string(t);

    // Element Jacobians, determinants, affinity check, DOF coordinates
    P.el_jac.assign((size_t)K * 9, 0.0);
    P.el_detj.assign(K, 0.0);
    P.dof_xyz.assign((size_t)K * np * 3, 0.0);
    P.el_curved.assign(K, 0);
    for (int e = 0; e < K; ++e) {
        const int *en = &m.el_nodes[(size_t)e * np];
        const double *x0 = X(en[0]);
        double jac[3][3] = {};
        for (int u = 0; u < dim; ++u) {
            const double *xu = X(en[u + 1]);
            for (int k = 0; k < 3; ++k) jac[u][k] = xu[k] - x0[k];
        }
        double h = 0;
        for (int u = 0; u < dim; ++u) h = std::max(h, norm3(jac[u]));
        if (dim == 2) {
            double c[3];
            cross3(jac[0], jac[1], c);
            P.el_detj[e] = norm3(c);
            complete_jacobian(2, jac);
        } else {
            double c[3];
            cross3(jac[1], jac[2], c);
            P.el_detj[e] = jac[0][0] * c[0] + jac[0][1] * c[1] + jac[0][2] * c[2];
        }
        if (!(P.el_detj[e] > 0)) return "degenerate or inverted element " + std::to_string(e);
        for (int u = 0; u < 3; ++u)
            for (int k = 0; k < 3; ++k) P.el_jac[(size_t)e * 9 + u * 3 + k] = jac[u][k];
        // curved: some node is off the affine image of the reference lattice
        // by more than 1e-11 of the element size
        double dev = 0;
        for (int i = 0; i < np; ++i) {
            const double *xi = X(en[i]);
            for (int k = 0; k < 3; ++k) {
                double a = x0[k];
                for (int u = 0; u < dim; ++u) a += jac[u][k] * re.r[i * 3 + u];
                dev = std::max(dev, std::fabs(a - xi[k]));
                P.dof_xyz[((size_t)e * np + i) * 3 + k] = xi[k];
            }
        }
        if (dev > 1e-11 * h) {
            P.el_curved[e] = 1;
            ++P.ncurved;
        }
    }
    if (P.ncurved > 0) {
        std::string err = element_points(m, re, X, P);
        if (!err.empty()) return err;
    }

    // Unique faces in first-occurrence order
    std::unordered_map<std::vector<int>, int, VecHash> face_of;
    face_of.reserve((size_t)K * nf);
    P.el_f_ids.assign((size_t)K * nf, -1);
    std::vector<std::vector<int>> nbrs;
    std::vector<int> key(nfp);
    for (int e = 0; e < K; ++e)
        for (int lf = 0; lf < nf; ++lf) {
            for (int k = 0; k < nfp; ++k) key[k] = m.el_nodes[(size_t)e * np + re.fmask[lf * nfp + k]];
            std::vector<int> sk = key;
            std::sort(sk.begin(), sk.end());
            auto it = face_of.find(sk);
            int f;
            if (it == face_of.end()) {
                f = (int)nbrs.size();
                face_of.emplace(std::move(sk), f);
                nbrs.push_back({});
                P.f_node_tags.insert(P.f_node_tags.end(), key.begin(), key.end());
            } else {
                f = it->second;
            }
            P.el_f_ids[(size_t)e * nf + lf] = f;
            nbrs[f].push_back(e);
        }
    const int F = (int)nbrs.size();
    P.F = F;
    P.f_nbr.assign((size_t)F * 2, -1);
    P.f_is_bnd.assign(F, 0);
    for (int f = 0; f < F; ++f) {
        if (nbrs[f].size() > 2) return "non-manifold face " + std::to_string(f);
        // a face shared twice by the same element cannot happen in a valid mesh
        P.f_nbr[f * 2] = nbrs[f][0];
        if (nbrs[f].size() == 2) P.f_nbr[f * 2 + 1] = nbrs[f][1];
        P.f_is_bnd[f] = nbrs[f].size() < 2;
    }
    // face node -> element node by tag
    P.f_n_to_el_n.assign((size_t)F * nfp * 2, -1);
    for (int f = 0; f < F; ++f)
        for (int s = 0; s < 2; ++s) {
            int e = P.f_nbr[f * 2 + s];
            if (e < 0) continue;
            const int *en = &m.el_nodes[(size_t)e * np];
            for (int k = 0; k < nfp; ++k) {
                int tag = P.f_node_tags[(size_t)f * nfp + k];
                int found = -1;
                for (int i = 0; i < np; ++i)
                    if (en[i] == tag) { found = i; break; }
                if (found < 0) return "face node not found in neighbour element";
                P.f_n_to_el_n[((size_t)f * nfp + k) * 2 + s] = found;
            }
        }

    // Face Jacobian determinant and normal at the first face quadrature point
    P.f_detj.assign(F, 0.0);
    P.f_normal.assign((size_t)F * 3, 0.0);
    for (int f = 0; f < F; ++f) {
        const int *fn = &P.f_node_tags[(size_t)f * nfp];
        const double *x0 = X(fn[0]);
        double jac[3][3] = {};
        if (dim == 2) {
            const double *x1 = X(fn[1]);
            for (int k = 0; k < 3; ++k) jac[0][k] = 0.5 * (x1[k] - x0[k]);
            P.f_detj[f] = norm3(jac[0]);
            complete_jacobian(1, jac);
        } else {
            const double *x1 = X(fn[1]), *x2 = X(fn[2]);
            for (int k = 0; k < 3; ++k) { jac[0][k] = x1[k] - x0[k]; jac[1][k] = x2[k] - x0[k]; }
            double c[3];
            cross3(jac[0], jac[1], c);
            P.f_detj[f] = norm3(c);
            complete_jacobian(2, jac);
        }
        // Solve A g = dphi/du with A[u][x] = jac[u][x] restricted to dim x dim
        double A[9];
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim; ++c) A[r * dim + c] = jac[r][c];
        double g0[3] = {0, 0, 0}, g1[3] = {0, 0, 0};
        g0[0] = re.dphi0_first[0];
        g1[0] = re.dphi1_first[0];
        if (dim == 3) { g0[1] = re.dphi0_first[1]; g1[1] = re.dphi1_first[1]; }
        if (!lu_solve(A, g0, dim) || !lu_solve(A, g1, dim)) return "singular face Jacobian";
        double n[3];
        if (dim == 2) {
            double z[3] = {0, 0, -1};
            double gg[3] = {g0[0], g0[1], 0};
            cross3(gg, z, n);
        } else {
            cross3(g0, g1, n);
        }
        double nn = norm3(n);
        for (int k = 0; k < 3; ++k) P.f_normal[(size_t)f * 3 + k] = n[k] / nn;
    }

    if (P.ncurved > 0) {
        std::string err = face_points(re, X, P);
        if (!err.empty()) return err;
    }

    // Orientation of each element face relative to the face normal
    P.el_f_orient.assign((size_t)K * nf, 1);
    for (int e = 0; e < K; ++e) {
        const int *en = &m.el_nodes[(size_t)e * np];
        double bc[3] = {0, 0, 0};
        for (int v = 0; v <= dim; ++v)
            for (int k = 0; k < 3; ++k) bc[k] += X(en[v])[k];
        for (int k = 0; k < 3; ++k) bc[k] /= (dim + 1);
        for (int lf = 0; lf < nf; ++lf) {
            const double *xf = X(en[re.fmask[lf * nfp]]);
            int f = P.el_f_ids[(size_t)e * nf + lf];
            double dot = 0;
            for (int k = 0; k < 3; ++k) dot += (xf[k] - bc[k]) * P.f_normal[(size_t)f * 3 + k];
            P.el_f_orient[(size_t)e * nf + lf] = (dot >= 0) ? 1 : -1;
        }
    }
    // Neighbour reordering: its guard compares the number of faces with 2, so
    // it only acts on two-face meshes (Mesh.cpp:307).
    if (F == 2) {
        for (int f = 0; f < F; ++f) {
            int e0 = P.f_nbr[f * 2];
            int elf = 0;
            for (int lf = 0; lf < nf; ++lf)
                if (P.el_f_ids[(size_t)e0 * nf + lf] == f) elf = lf;
            if (P.f_nbr[f * 2 + 1] >= 0 && P.el_f_orient[(size_t)e0 * nf + elf] <= 0) {
                std::swap(P.f_nbr[f * 2], P.f_nbr[f * 2 + 1]);
                for (int k = 0; k < nfp; ++k)
                    std::swap(P.f_n_to_el_n[((size_t)f * nfp + k) * 2], P.f_n_to_el_n[((size_t)f * nfp + k) * 2 + 1]);
            }
        }
    }
    // Boundary faces: outward normal, orientation +1
    for (int f = 0; f < F; ++f) {
        if (!P.f_is_bnd[f]) continue;
        int e0 = P.f_nbr[f * 2];
        for (int lf = 0; lf < nf; ++lf) {
            if (P.el_f_ids[(size_t)e0 * nf + lf] != f) continue;
            int o = P.el_f_orient[(size_t)e0 * nf + lf];
            for (int k = 0; k < 3; ++k) P.f_normal[(size_t)f * 3 + k] *= o;
            for (size_t k = 0; k < (size_t)P.ngf * 3 && P.ncurved > 0; ++k)
                P.f_normal_qp[(size_t)f * P.ngf * 3 + k] *= o;
            P.el_f_orient[(size_t)e0 * nf + lf] = 1;
        }
    }
    // Boundary types
    P.f_bc.assign(F, 0);
    for (auto &pb : physical_bcs) {
        const PhysGroup *g = nullptr;
        for (auto &pg : m.phys)
            if (pg.dim == dim - 1 && pg.tag == pb.first) g = &pg;
        if (!g) continue;
        for (int f = 0; f < F; ++f) {
            if (!P.f_is_bnd[f]) continue;
            int first = P.f_node_tags[(size_t)f * nfp];
            if (std::binary_search(g->nodes.begin(), g->nodes.end(), first)) P.f_bc[f] = pb.second ? 1 : 0;
        }
    }
    return "";
}

}  // namespace dg
