// Reference-semantics mesh precompute for affine simplices.
#include "precompute.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <unordered_map>

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

}  // namespace

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

    // node tag -> coordinates
    int maxtag = 0;
    for (int t : m.node_tags) maxtag = std::max(maxtag, t);
    std::vector<int> idx(maxtag + 1, -1);
    for (size_t i = 0; i < m.node_tags.size(); ++i) idx[m.node_tags[i]] = (int)i;
    auto X = [&](int tag) -> const double * {
        if (tag < 0 || tag > maxtag || idx[tag] < 0) return nullptr;
        return &m.xyz[idx[tag] * 3];
    };
    for (int t : m.el_nodes)
        if (!X(t)) return "element references an unknown node tag " + std::to_string(t);

    // Element Jacobians, determinants, affinity check, DOF coordinates
    P.el_jac.assign((size_t)K * 9, 0.0);
    P.el_detj.assign(K, 0.0);
    P.dof_xyz.assign((size_t)K * np * 3, 0.0);
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
        for (int i = 0; i < np; ++i) {
            const double *xi = X(en[i]);
            double dev = 0;
            for (int k = 0; k < 3; ++k) {
                double a = x0[k];
                for (int u = 0; u < dim; ++u) a += jac[u][k] * re.r[i * 3 + u];
                dev = std::max(dev, std::fabs(a - xi[k]));
                P.dof_xyz[((size_t)e * np + i) * 3 + k] = xi[k];
            }
            if (dev > 1e-9 * h) return "curved (non-affine) element " + std::to_string(e) + " is not supported";
        }
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
