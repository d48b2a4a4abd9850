// Reference simplex elements: node lattices, orthonormal basis, DG operators.
#include "refel.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <stdexcept>

namespace dg {

namespace {

const int kTriEdges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kTetEdges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
const int kTetFaces[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};

Bary lerp(const Bary &a, const Bary &b, int k, int m) {
    Bary r{};
    for (int i = 0; i < 4; ++i) r[i] = a[i] + (b[i] - a[i]) / m * k;
    return r;
}

// Vertex of the inner simplex: v + sum_{w != v} (w - v)/m
Bary inner_vertex(const Bary *verts, int nv, int which, int m) {
    Bary r = verts[which];
    for (int w = 0; w < nv; ++w) {
        if (w == which) continue;
        for (int i = 0; i < 4; ++i) r[i] += (verts[w][i] - verts[which][i]) / m;
    }
    return r;
}

void line_nodes(const Bary &a, const Bary &b, int m, std::vector<Bary> &out) {
    if (m == 0) { out.push_back(a); return; }
    out.push_back(a);
    out.push_back(b);
    for (int k = 1; k < m; ++k) out.push_back(lerp(a, b, k, m));
}

void tri_nodes(const Bary *v, int m, std::vector<Bary> &out) {
    if (m == 0) { out.push_back(v[0]); return; }
    for (int i = 0; i < 3; ++i) out.push_back(v[i]);
    for (auto &e : kTriEdges)
        for (int k = 1; k < m; ++k) out.push_back(lerp(v[e[0]], v[e[1]], k, m));
    if (m >= 3) {
        Bary in[3];
        for (int i = 0; i < 3; ++i) in[i] = inner_vertex(v, 3, i, m);
        tri_nodes(in, m - 3, out);
    }
}

void tet_nodes(const Bary *v, int m, std::vector<Bary> &out) {
    if (m == 0) { out.push_back(v[0]); return; }
    for (int i = 0; i < 4; ++i) out.push_back(v[i]);
    for (auto &e : kTetEdges)
        for (int k = 1; k < m; ++k) out.push_back(lerp(v[e[0]], v[e[1]], k, m));
    if (m >= 3) {
        for (auto &f : kTetFaces) {
            Bary fv[3] = {v[f[0]], v[f[1]], v[f[2]]};
            Bary in[3];
            for (int i = 0; i < 3; ++i) in[i] = inner_vertex(fv, 3, i, m);
            tri_nodes(in, m - 3, out);
        }
    }
    if (m >= 4) {
        Bary in[4];
        for (int i = 0; i < 4; ++i) in[i] = inner_vertex(v, 4, i, m);
        tet_nodes(in, m - 4, out);
    }
}

// Orthonormal Jacobi polynomial P_n^{(a,b)} on [-1,1] (weight (1-x)^a (1+x)^b).
double jacobi_p(double x, double alpha, double beta, int n) {
    double g0 = std::pow(2.0, alpha + beta + 1) / (alpha + beta + 1) * std::tgamma(alpha + 1) *
                std::tgamma(beta + 1) / std::tgamma(alpha + beta + 1);
    double p0 = 1.0 / std::sqrt(g0);
    if (n == 0) return p0;
    double g1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * g0;
    double p1 = ((alpha + beta + 2) * x / 2 + (alpha - beta) / 2) / std::sqrt(g1);
    if (n == 1) return p1;
    double aold = 2 / (2 + alpha + beta) * std::sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3));
    double pm1 = p0, pc = p1;
    for (int i = 1; i < n; ++i) {
        double h1 = 2 * i + alpha + beta;
        double anew = 2 / (h1 + 2) *
                      std::sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha) * (i + 1 + beta) /
                                (h1 + 1) / (h1 + 3));
        double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2);
        double pn = (-aold * pm1 + (x - bnew) * pc) / anew;
        pm1 = pc;
        pc = pn;
        aold = anew;
    }
    return pc;
}

double grad_jacobi_p(double x, double alpha, double beta, int n) {
    if (n == 0) return 0.0;
    return std::sqrt(n * (n + alpha + beta + 1)) * jacobi_p(x, alpha + 1, beta + 1, n - 1);
}

struct Mode { int i, j, k; };

std::vector<Mode> modes(int d, int p) {
    std::vector<Mode> m;
    if (d == 1) {
        for (int i = 0; i <= p; ++i) m.push_back({i, 0, 0});
    } else if (d == 2) {
        for (int i = 0; i <= p; ++i)
            for (int j = 0; j + i <= p; ++j) m.push_back({i, j, 0});
    } else {
        for (int i = 0; i <= p; ++i)
            for (int j = 0; i + j <= p; ++j)
                for (int k = 0; i + j + k <= p; ++k) m.push_back({i, j, k});
    }
    return m;
}

// Basis on the [-1,1] "rst" simplex; gradient wrt r,s,t.
void ortho_rst(int d, int p, const double *rst, double *psi, double *dpsi) {
    auto ms = modes(d, p);
    if (d == 1) {
        for (size_t n = 0; n < ms.size(); ++n) {
            psi[n] = jacobi_p(rst[0], 0, 0, ms[n].i);
            if (dpsi) {
                dpsi[n * 3 + 0] = grad_jacobi_p(rst[0], 0, 0, ms[n].i);
                dpsi[n * 3 + 1] = dpsi[n * 3 + 2] = 0;
            }
        }
        return;
    }
    if (d == 2) {
        double r = rst[0], s = rst[1];
        double a = (s != 1.0) ? 2 * (1 + r) / (1 - s) - 1 : -1.0;
        double b = s;
        for (size_t n = 0; n < ms.size(); ++n) {
            int i = ms[n].i, j = ms[n].j;
            double fa = jacobi_p(a, 0, 0, i), gb = jacobi_p(b, 2 * i + 1, 0, j);
            psi[n] = std::sqrt(2.0) * fa * gb * std::pow(1 - b, i);
            if (!dpsi) continue;
            double dfa = grad_jacobi_p(a, 0, 0, i), dgb = grad_jacobi_p(b, 2 * i + 1, 0, j);
            double dr = dfa * gb;
            if (i > 0) dr *= std::pow(0.5 * (1 - b), i - 1);
            double ds = dfa * (gb * (0.5 * (1 + a)));
            if (i > 0) ds *= std::pow(0.5 * (1 - b), i - 1);
            double tmp = dgb * std::pow(0.5 * (1 - b), i);
            if (i > 0) tmp -= 0.5 * i * gb * std::pow(0.5 * (1 - b), i - 1);
            ds += fa * tmp;
            double sc = std::pow(2.0, i + 0.5);
            dpsi[n * 3 + 0] = dr * sc;
            dpsi[n * 3 + 1] = ds * sc;
            dpsi[n * 3 + 2] = 0;
        }
        return;
    }
    double r = rst[0], s = rst[1], t = rst[2];
    double a = (s + t != 0.0) ? 2 * (1 + r) / (-s - t) - 1 : -1.0;
    double b = (t != 1.0) ? 2 * (1 + s) / (1 - t) - 1 : -1.0;
    double c = t;
    for (size_t n = 0; n < ms.size(); ++n) {
        int i = ms[n].i, j = ms[n].j, k = ms[n].k;
        double fa = jacobi_p(a, 0, 0, i), gb = jacobi_p(b, 2 * i + 1, 0, j);
        double hc = jacobi_p(c, 2 * (i + j) + 2, 0, k);
        psi[n] = 2 * std::sqrt(2.0) * fa * gb * std::pow(1 - b, i) * hc * std::pow(1 - c, i + j);
        if (!dpsi) continue;
        double dfa = grad_jacobi_p(a, 0, 0, i), dgb = grad_jacobi_p(b, 2 * i + 1, 0, j);
        double dhc = grad_jacobi_p(c, 2 * (i + j) + 2, 0, k);
        double vr = dfa * (gb * hc);
        if (i > 0) vr *= std::pow(0.5 * (1 - b), i - 1);
        if (i + j > 0) vr *= std::pow(0.5 * (1 - c), i + j - 1);
        double vs = 0.5 * (1 + a) * vr;
        double tmp = dgb * std::pow(0.5 * (1 - b), i);
        if (i > 0) tmp += -0.5 * i * (gb * std::pow(0.5 * (1 - b), i - 1));
        if (i + j > 0) tmp *= std::pow(0.5 * (1 - c), i + j - 1);
        tmp = fa * (tmp * hc);
        vs += tmp;
        double vt = 0.5 * (1 + a) * vr + 0.5 * (1 + b) * tmp;
        tmp = dhc * std::pow(0.5 * (1 - c), i + j);
        if (i + j > 0) tmp -= 0.5 * (i + j) * (hc * std::pow(0.5 * (1 - c), i + j - 1));
        tmp = fa * (gb * tmp);
        tmp *= std::pow(0.5 * (1 - b), i);
        vt += tmp;
        double sc = std::pow(2.0, 2 * i + j + 1.5);
        dpsi[n * 3 + 0] = vr * sc;
        dpsi[n * 3 + 1] = vs * sc;
        dpsi[n * 3 + 2] = vt * sc;
    }
}

// gmsh reference coordinates -> rst coordinates
void to_rst(int d, const double *x, double *rst) {
    if (d == 1) { rst[0] = x[0]; rst[1] = rst[2] = 0; return; }
    for (int i = 0; i < 3; ++i) rst[i] = (i < d) ? 2 * x[i] - 1 : 0;
}
double coord_scale(int d) { return d == 1 ? 1.0 : 2.0; }

void bary_to_ref(int d, int order, const Bary &b, double *x) {
    x[0] = x[1] = x[2] = 0;
    if (d == 1) { x[0] = double(b[1] - b[0]) / order; return; }
    for (int i = 0; i < d; ++i) x[i] = double(b[i + 1]) / order;
}

struct VCache { std::vector<double> vinv; };
std::mutex g_cache_mu;
std::map<std::pair<int, int>, VCache> g_cache;

const std::vector<double> &vandermonde_inverse(int d, int p) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto key = std::make_pair(d, p);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) return it->second.vinv;
    auto nodes = simplex_lattice(d, p);
    int n = (int)nodes.size();
    std::vector<double> V(n * n);
    std::vector<double> psi(n);
    for (int i = 0; i < n; ++i) {
        double x[3], rst[3];
        bary_to_ref(d, p, nodes[i], x);
        to_rst(d, x, rst);
        ortho_rst(d, p, rst, psi.data(), nullptr);
        for (int m = 0; m < n; ++m) V[i * n + m] = psi[m];
    }
    if (!lu_inverse(V, n)) throw std::runtime_error("singular Vandermonde");
    g_cache[key].vinv = V;
    return g_cache[key].vinv;
}

double gauss_legendre_min_root(int n) {
    // smallest root of P_n by Newton from the standard asymptotic guess
    double x = -std::cos(M_PI * (0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
        double p0 = 1, p1 = x;
        for (int k = 2; k <= n; ++k) {
            double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        double dp = n * (x * p1 - p0) / (x * x - 1);
        double dx = p1 / dp;
        x -= dx;
        if (std::fabs(dx) < 1e-16) break;
    }
    return x;
}

}  // namespace

int simplex_np(int d, int p) {
    if (d == 1) return p + 1;
    if (d == 2) return (p + 1) * (p + 2) / 2;
    return (p + 1) * (p + 2) * (p + 3) / 6;
}

std::vector<Bary> simplex_lattice(int dim, int order) {
    std::vector<Bary> out;
    Bary v[4] = {};
    for (int i = 0; i <= dim; ++i) { v[i] = Bary{0, 0, 0, 0}; v[i][i] = order; }
    if (dim == 1) line_nodes(v[0], v[1], order, out);
    else if (dim == 2) tri_nodes(v, order, out);
    else tet_nodes(v, order, out);
    return out;
}

std::vector<Bary> face_lattice_on(int fdim, const Bary *verts, int order) {
    std::vector<Bary> out;
    if (fdim == 1) line_nodes(verts[0], verts[1], order, out);
    else tri_nodes(verts, order, out);
    return out;
}

bool lu_inverse(std::vector<double> &A, int n) {
    std::vector<double> inv(n * n, 0.0);
    for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
    std::vector<double> a = A;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
        if (a[piv * n + c] == 0.0) return false;
        if (piv != c)
            for (int k = 0; k < n; ++k) {
                std::swap(a[c * n + k], a[piv * n + k]);
                std::swap(inv[c * n + k], inv[piv * n + k]);
            }
        double d = 1.0 / a[c * n + c];
        for (int k = 0; k < n; ++k) { a[c * n + k] *= d; inv[c * n + k] *= d; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = a[r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                a[r * n + k] -= f * a[c * n + k];
                inv[r * n + k] -= f * inv[c * n + k];
            }
        }
    }
    A = inv;
    return true;
}

bool lu_solve(const double *A, double *b, int n) {
    std::vector<double> a(A, A + n * n);
    std::vector<int> p(n);
    for (int i = 0; i < n; ++i) p[i] = i;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
        if (a[piv * n + c] == 0.0) return false;
        if (piv != c) {
            for (int k = 0; k < n; ++k) std::swap(a[c * n + k], a[piv * n + k]);
            std::swap(b[c], b[piv]);
        }
        for (int r = c + 1; r < n; ++r) {
            double f = a[r * n + c] / a[c * n + c];
            for (int k = c; k < n; ++k) a[r * n + k] -= f * a[c * n + k];
            b[r] -= f * b[c];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = b[r];
        for (int k = r + 1; k < n; ++k) s -= a[r * n + k] * b[k];
        b[r] = s / a[r * n + r];
    }
    return true;
}

void ortho_basis(int d, int p, const double *x, double *psi, double *dpsi) {
    double rst[3];
    to_rst(d, x, rst);
    ortho_rst(d, p, rst, psi, dpsi);
    if (dpsi) {
        int n = simplex_np(d, p);
        double sc = coord_scale(d);
        for (int i = 0; i < n * 3; ++i) dpsi[i] *= sc;
    }
}

void lagrange_eval(int d, int p, const double *x, double *phi, double *dphi) {
    const auto &vinv = vandermonde_inverse(d, p);
    int n = simplex_np(d, p);
    std::vector<double> psi(n), dpsi(3 * n);
    ortho_basis(d, p, x, psi.data(), dphi ? dpsi.data() : nullptr);
    for (int k = 0; k < n; ++k) {
        double v = 0, g0 = 0, g1 = 0, g2 = 0;
        for (int m = 0; m < n; ++m) {
            double c = vinv[m * n + k];
            v += psi[m] * c;
            if (dphi) { g0 += dpsi[m * 3] * c; g1 += dpsi[m * 3 + 1] * c; g2 += dpsi[m * 3 + 2] * c; }
        }
        if (phi) phi[k] = v;
        if (dphi) { dphi[k * 3] = g0; dphi[k * 3 + 1] = g1; dphi[k * 3 + 2] = g2; }
    }
}

RefElement make_refel(int dim, int order) {
    if (dim < 2 || dim > 3) throw std::runtime_error("dimension must be 2 or 3");
    if (order < 1 || order > 5) throw std::runtime_error("order must be in 1..5");
    RefElement re;
    re.dim = dim;
    re.order = order;
    re.nodes = simplex_lattice(dim, order);
    re.np = (int)re.nodes.size();
    re.nf = dim + 1;
    re.nfp = simplex_np(dim - 1, order);
    re.nperm = (dim == 2) ? 2 : 6;
    const int np = re.np, nfp = re.nfp, p = order;

    re.r.assign(np * 3, 0.0);
    for (int i = 0; i < np; ++i) bary_to_ref(dim, p, re.nodes[i], &re.r[i * 3]);

    // Faces and face masks
    Bary V[4];
    for (int i = 0; i < 4; ++i) { V[i] = Bary{0, 0, 0, 0}; if (i <= dim) V[i][i] = p; }
    re.face_verts.assign(re.nf * 3, -1);
    re.fmask.assign(re.nf * nfp, -1);
    for (int f = 0; f < re.nf; ++f) {
        Bary fv[3];
        int nv = dim;  // vertices per face
        for (int k = 0; k < nv; ++k) {
            int vid = (dim == 2) ? kTriEdges[f][k] : kTetFaces[f][k];
            re.face_verts[f * 3 + k] = vid;
            fv[k] = V[vid];
        }
        auto fl = face_lattice_on(dim - 1, fv, p);
        for (int k = 0; k < nfp; ++k) {
            auto it = std::find(re.nodes.begin(), re.nodes.end(), fl[k]);
            if (it == re.nodes.end()) throw std::runtime_error("face node not found");
            re.fmask[f * nfp + k] = int(it - re.nodes.begin());
        }
    }

    // Face symmetries
    {
        Bary A[3];
        int nv = dim;
        for (int k = 0; k < 3; ++k) { A[k] = Bary{0, 0, 0, 0}; if (k < nv) A[k][k] = p; }
        std::vector<std::array<int, 3>> perms;
        if (dim == 2) perms = {{0, 1, 2}, {1, 0, 2}};
        else perms = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
        auto gid = face_lattice_on(dim - 1, A, p);
        re.perm.assign(re.nperm * nfp, -1);
        re.perm_verts.assign(re.nperm * 3, 0);
        for (int pi = 0; pi < re.nperm; ++pi) {
            Bary B[3];
            for (int k = 0; k < nv; ++k) B[k] = A[perms[pi][k]];
            auto gp = face_lattice_on(dim - 1, B, p);
            for (int k = 0; k < 3; ++k) re.perm_verts[pi * 3 + k] = perms[pi][k];
            for (int k = 0; k < nfp; ++k) {
                auto it = std::find(gp.begin(), gp.end(), gid[k]);
                re.perm[pi * nfp + k] = int(it - gp.begin());
            }
        }
        // face node reference coordinates (face simplex)
        re.face_r.assign(nfp * 2, 0.0);
        for (int k = 0; k < nfp; ++k) {
            double x[3];
            bary_to_ref(dim - 1, p, gid[k], x);
            re.face_r[k * 2] = x[0];
            re.face_r[k * 2 + 1] = x[1];
        }
    }

    // Vandermonde and operators
    const auto &vinv = vandermonde_inverse(dim, p);
    std::vector<double> Vm(np * np), Vg(3 * np * np);
    {
        std::vector<double> psi(np), dpsi(3 * np);
        for (int i = 0; i < np; ++i) {
            ortho_basis(dim, p, &re.r[i * 3], psi.data(), dpsi.data());
            for (int m = 0; m < np; ++m) {
                Vm[i * np + m] = psi[m];
                for (int u = 0; u < 3; ++u) Vg[(u * np + i) * np + m] = dpsi[m * 3 + u];
            }
        }
    }
    // mass inverse = s^d V V^T (orthonormality on the rst simplex)
    double sd = std::pow(coord_scale(dim), dim);
    re.mass_inv.assign(np * np, 0.0);
    for (int i = 0; i < np; ++i)
        for (int j = 0; j < np; ++j) {
            double s = 0;
            for (int m = 0; m < np; ++m) s += Vm[i * np + m] * Vm[j * np + m];
            re.mass_inv[i * np + j] = s * sd;
        }
    re.mass = re.mass_inv;
    if (!lu_inverse(re.mass, np)) throw std::runtime_error("singular mass");
    // nodal derivative Dn_u = Vg_u * Vinv ; D_u = Minv Dn_u^T M
    re.D.assign(dim * np * np, 0.0);
    for (int u = 0; u < dim; ++u) {
        std::vector<double> Dn(np * np, 0.0), T(np * np, 0.0);
        for (int i = 0; i < np; ++i)
            for (int j = 0; j < np; ++j) {
                double s = 0;
                for (int m = 0; m < np; ++m) s += Vg[(u * np + i) * np + m] * vinv[m * np + j];
                Dn[i * np + j] = s;
            }
        // T = Dn^T M
        for (int i = 0; i < np; ++i)
            for (int j = 0; j < np; ++j) {
                double s = 0;
                for (int k = 0; k < np; ++k) s += Dn[k * np + i] * re.mass[k * np + j];
                T[i * np + j] = s;
            }
        for (int i = 0; i < np; ++i)
            for (int j = 0; j < np; ++j) {
                double s = 0;
                for (int k = 0; k < np; ++k) s += re.mass_inv[i * np + k] * T[k * np + j];
                re.D[(u * np + i) * np + j] = s;
            }
    }
    // face mass on the reference face simplex
    {
        int fd = dim - 1;
        const auto &fvinv = vandermonde_inverse(fd, p);
        // Mf^-1 = s^fd Vf Vf^T ; Vf = inverse of fvinv
        std::vector<double> Vf = fvinv;
        lu_inverse(Vf, nfp);
        double sfd = std::pow(coord_scale(fd), fd);
        std::vector<double> mfi(nfp * nfp);
        for (int i = 0; i < nfp; ++i)
            for (int j = 0; j < nfp; ++j) {
                double s = 0;
                for (int m = 0; m < nfp; ++m) s += Vf[i * nfp + m] * Vf[j * nfp + m];
                mfi[i * nfp + j] = s * sfd;
            }
        re.fmass = mfi;
        lu_inverse(re.fmass, nfp);
    }
    // lift
    re.lift.assign(re.nf * np * nfp, 0.0);
    for (int f = 0; f < re.nf; ++f)
        for (int i = 0; i < np; ++i)
            for (int k = 0; k < nfp; ++k) {
                double s = 0;
                for (int l = 0; l < nfp; ++l)
                    s += re.mass_inv[i * np + re.fmask[f * nfp + l]] * re.fmass[l * nfp + k];
                re.lift[(f * np + i) * nfp + k] = s;
            }

    // First point of the face Gauss(2p) rule and face basis derivatives there
    if (dim == 2) {
        re.face_first_pt[0] = gauss_legendre_min_root(p + 1);
    } else {
        static const double tri_first[6][2] = {
            {0, 0}, {1.0 / 6.0, 1.0 / 6.0}, {0.445948490915965, 0.445948490915965},
            {0.249286745170910, 0.249286745170910}, {1.0 / 3.0, 1.0 / 3.0}, {1.0 / 3.0, 1.0 / 3.0}};
        re.face_first_pt[0] = tri_first[p][0];
        re.face_first_pt[1] = tri_first[p][1];
    }
    {
        std::vector<double> dphi(3 * nfp);
        double x[3] = {re.face_first_pt[0], re.face_first_pt[1], 0};
        lagrange_eval(dim - 1, p, x, nullptr, dphi.data());
        re.dphi0_first[0] = dphi[0]; re.dphi0_first[1] = dphi[1];
        re.dphi1_first[0] = dphi[3]; re.dphi1_first[1] = dphi[4];
    }
    return re;
}

}  // namespace dg
