// ============================================================================
// TEST INFRASTRUCTURE ONLY - the CPU oracle of the DG acoustic RK4 path.
//
// Only the tests, the smoke check and bench.py's CPU-baseline leg may load
// this library.  It is never part of the product path.
//
// What it is: a faithful C++/OpenMP restatement of the reference's hot path
// and of the set-up it reads:
//   Mesh::Mesh            src/Mesh.cpp:20-435   (OMesh::OMesh)
//   getUniqueFaceNodeTags src/Mesh.cpp:679-713  (semantics kept, hashed search)
//   precomputeMassMatrix  src/Mesh.cpp:440-466
//   getElStiffVector      src/Mesh.cpp:476-489
//   precomputeFlux        src/Mesh.cpp:500-539  (nested OpenMP region kept)
//   getElFlux             src/Mesh.cpp:548-557
//   updateFlux            src/Mesh.cpp:569-674
//   numStep               src/solver.cpp:35-52
//   rungeKutta loop body  src/solver.cpp:197-210, 247-285
//   forwardEuler body     src/solver.cpp:138-153
// with the same loops, data layouts (vector-of-vector Flux, per-element
// gradient tables, per-element inverse mass matrices) and OpenMP pragmas.
//
// The reference gets its element data from the gmsh SDK 4.1.4 and its small
// linear algebra from Eigen 3.3.7, neither of which is in the reference
// checkout.  Their published behaviour is restated here:
//   * Lagrange basis functions as monomials times the inverse monomial
//     Vandermonde (gmsh's polynomial basis), gmsh node ordering;
//   * "Gauss<2p>" rules: oracle/quadrature_tables.inc (Gauss-Legendre lines,
//     Dunavant triangles, Keast-type tetrahedra);
//   * getJacobians: J = sum_k x_k dphi_k/du at each point, completed for
//     lines (b = (a1,-a0,0) or (0,a2,-a1), c = a x b) and triangles
//     (c = row0 x row1), determinant |J0|, |J0 x J1| or det J;
//   * getBarycenters (primary nodes), getElementEdgeNodes/FaceNodes,
//     getNodesForPhysicalGroup;
//   * Eigen: partial-pivot LU solve and inverse, dot, cross, normalize.
//
// PARITY UNPINNED: the reference has no tests, golden vectors or known-answer
// data for this path, and it cannot be built here (it needs the gmsh SDK and
// Eigen).  This oracle is checked against analytic known answers instead
// (tests/test_oracle.py).
// ============================================================================
#include <omp.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "quadrature_tables.inc"

namespace oracle {

// ---------------------------------------------------------------------------
// Small linear algebra (Eigen restatement)
// ---------------------------------------------------------------------------
namespace la {
// A is column-major n x n (Eigen::Map<MatrixXd>), B overwritten by A^-1 B.
void solve(const double *A, double *B, int n) {
    std::vector<double> a(A, A + n * n);  // a[c*n + r]
    std::vector<int> piv(n);
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(a[k * n + r]) > std::fabs(a[k * n + p])) p = r;
        piv[k] = p;
        if (p != k) {
            for (int c = 0; c < n; ++c) std::swap(a[c * n + k], a[c * n + p]);
            std::swap(B[k], B[p]);
        }
        double d = a[k * n + k];
        for (int r = k + 1; r < n; ++r) {
            double l = a[k * n + r] / d;
            a[k * n + r] = l;
            for (int c = k + 1; c < n; ++c) a[c * n + r] -= l * a[c * n + k];
            B[r] -= l * B[k];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = B[r];
        for (int c = r + 1; c < n; ++c) s -= a[c * n + r] * B[c];
        B[r] = s / a[r * n + r];
    }
}
// In-place inverse of a square matrix (storage order irrelevant: inverse of
// the transpose is the transpose of the inverse).
void inverse(double *A, int n) {
    std::vector<double> inv(n * n, 0.0), col(n);
    for (int j = 0; j < n; ++j) {
        std::fill(col.begin(), col.end(), 0.0);
        col[j] = 1.0;
        solve(A, col.data(), n);
        for (int i = 0; i < n; ++i) inv[j * n + i] = col[i];
    }
    std::copy(inv.begin(), inv.end(), A);
}
void normalize(double *A, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += A[i] * A[i];
    s = std::sqrt(s);
    for (int i = 0; i < n; ++i) A[i] /= s;
}
// y = beta*y + alpha*A*x with A column-major (Eigen::Map<MatrixXd> of a
// row-major array, i.e. the transpose of the stored matrix).
void linEq(const double *A, const double *X, double *Y, double alpha, double beta, int n) {
    std::vector<double> ax(n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) ax[r] += A[c * n + r] * X[c];
    for (int r = 0; r < n; ++r) Y[r] = beta * Y[r] + alpha * ax[r];
}
double dot(const double *A, const double *B, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += A[i] * B[i];
    return s;
}
void minus(double *A, const double *B, int n) {
    for (int i = 0; i < n; ++i) A[i] -= B[i];
}
void plusTimes(double *A, const double *B, double c, int n) {
    for (int i = 0; i < n; ++i) A[i] += c * B[i];
}
void cross(const double *A, const double *B, double *O) {
    O[0] = A[1] * B[2] - A[2] * B[1];
    O[1] = A[2] * B[0] - A[0] * B[2];
    O[2] = A[0] * B[1] - A[1] * B[0];
}
}  // namespace la

// ---------------------------------------------------------------------------
// gmsh restatement: reference elements, Lagrange bases, rules
// ---------------------------------------------------------------------------
typedef std::array<double, 3> P3;
// The reference-element lattice and the Lagrange basis are built in long
// double (x86-64: 64-bit significand; aarch64: IEEE binary128) and rounded to
// double once.  gmsh's monomial Vandermonde at equispaced nodes is badly
// conditioned at orders 4-5 (3D order 5: 56 x 56), so a double inverse and a
// double evaluation of sum_m c_m x^m lose several digits in cancellation;
// extended precision keeps the basis values and gradients at the rule points
// correct to double rounding, with the same monomial representation.
typedef long double LD;
typedef std::array<LD, 3> PL;

// Nodes of the order-p element on the given vertices (reference coordinates),
// gmsh order: vertices, edges (in edge direction), faces, interior.
template <class PT>
static void push_edge(std::vector<PT> &out, const PT &a, const PT &b, int p) {
    for (int k = 1; k < p; ++k) {
        typename PT::value_type t = typename PT::value_type(k) / p;
        out.push_back({a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1]), a[2] + t * (b[2] - a[2])});
    }
}
template <class PT>
static PT shrink(const PT *v, int nv, int which, int p) {
    // vertex of the inner simplex: v_w + sum_{o != w} (v_o - v_w)/p
    PT r = v[which];
    for (int o = 0; o < nv; ++o)
        if (o != which)
            for (int k = 0; k < 3; ++k) r[k] += (v[o][k] - v[which][k]) / p;
    return r;
}
template <class PT>
static void tri_points(std::vector<PT> &out, PT a, PT b, PT c, int p) {
    while (true) {
        if (p == 0) {
            out.push_back(a);
            return;
        }
        out.push_back(a);
        out.push_back(b);
        out.push_back(c);
        push_edge(out, a, b, p);
        push_edge(out, b, c, p);
        push_edge(out, c, a, p);
        if (p < 3) return;
        PT v[3] = {a, b, c};
        PT na = shrink(v, 3, 0, p), nb = shrink(v, 3, 1, p), nc = shrink(v, 3, 2, p);
        a = na; b = nb; c = nc;
        p -= 3;
    }
}
static const int kTetEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
static const int kTetFace[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};
static const int kTriEdge[3][2] = {{0, 1}, {1, 2}, {2, 0}};
template <class PT>
static void tet_points(std::vector<PT> &out, PT v0, PT v1, PT v2, PT v3, int p) {
    while (true) {
        PT v[4] = {v0, v1, v2, v3};
        if (p == 0) {
            out.push_back(v0);
            return;
        }
        for (int i = 0; i < 4; ++i) out.push_back(v[i]);
        for (auto &e : kTetEdge) push_edge(out, v[e[0]], v[e[1]], p);
        if (p >= 3)
            for (auto &f : kTetFace) {
                PT fv[3] = {v[f[0]], v[f[1]], v[f[2]]};
                tri_points(out, shrink(fv, 3, 0, p), shrink(fv, 3, 1, p), shrink(fv, 3, 2, p), p - 3);
            }
        if (p < 4) return;
        PT n0 = shrink(v, 4, 0, p), n1 = shrink(v, 4, 1, p), n2 = shrink(v, 4, 2, p), n3 = shrink(v, 4, 3, p);
        v0 = n0; v1 = n1; v2 = n2; v3 = n3;
        p -= 4;
    }
}

// In-place inverse (partial-pivot Gauss-Jordan) of a column-major n x n
// long double matrix; the Vandermonde of distinct lattice nodes is regular.
static void inverse_ld(std::vector<LD> &a, int n) {
    std::vector<LD> inv(n * n, 0.0L);
    for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0L;
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(a[k * n + r]) > std::fabs(a[k * n + p])) p = r;
        if (p != k)
            for (int c = 0; c < n; ++c) {
                std::swap(a[c * n + k], a[c * n + p]);
                std::swap(inv[c * n + k], inv[c * n + p]);
            }
        LD d = a[k * n + k];
        for (int c = 0; c < n; ++c) {
            a[c * n + k] /= d;
            inv[c * n + k] /= d;
        }
        for (int r = 0; r < n; ++r) {
            if (r == k) continue;
            LD l = a[k * n + r];
            if (l == 0.0L) continue;
            for (int c = 0; c < n; ++c) {
                a[c * n + r] -= l * a[c * n + k];
                inv[c * n + r] -= l * inv[c * n + k];
            }
        }
    }
    a.swap(inv);
}

struct Basis {
    int dim = 0, order = 0, n = 0;
    std::vector<P3> nodes;                 // reference coordinates (rounded)
    std::vector<std::array<int, 3>> mono;  // exponents
    std::vector<LD> coef;                  // [m][k]: phi_k = sum_m coef[m][k] mono_m
    void build(int d, int p) {
        dim = d;
        order = p;
        std::vector<PL> ln;
        if (d == 1) {
            ln.push_back({-1, 0, 0});
            ln.push_back({1, 0, 0});
            push_edge(ln, PL{-1, 0, 0}, PL{1, 0, 0}, p);
        } else if (d == 2) {
            tri_points(ln, PL{0, 0, 0}, PL{1, 0, 0}, PL{0, 1, 0}, p);
        } else {
            tet_points(ln, PL{0, 0, 0}, PL{1, 0, 0}, PL{0, 1, 0}, PL{0, 0, 1}, p);
        }
        n = (int)ln.size();
        nodes.resize(n);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) nodes[i][k] = (double)ln[i][k];
        mono.clear();
        for (int a = 0; a <= p; ++a)
            for (int b = 0; b <= (d >= 2 ? p - a : 0); ++b)
                for (int c = 0; c <= (d == 3 ? p - a - b : 0); ++c) mono.push_back({a, b, c});
        std::vector<LD> V(n * n);  // column-major V(i,m) = mono_m(x_i)
        for (int i = 0; i < n; ++i)
            for (int m = 0; m < n; ++m) V[m * n + i] = mono_val(m, ln[i].data());
        inverse_ld(V, n);  // V^-1 column-major: Vi(m,k) at [k*n + m]
        coef.assign(n * n, 0.0L);
        for (int m = 0; m < n; ++m)
            for (int k = 0; k < n; ++k) coef[m * n + k] = V[k * n + m];
    }
    static LD ipow(LD x, int e) {
        LD r = 1.0L;
        for (int i = 0; i < e; ++i) r *= x;
        return r;
    }
    LD mono_val(int m, const LD *x) const {
        return ipow(x[0], mono[m][0]) * ipow(x[1], mono[m][1]) * ipow(x[2], mono[m][2]);
    }
    LD mono_der(int m, int dir, const LD *x) const {
        int e = mono[m][dir];
        if (e == 0) return 0.0L;
        LD v = e;
        for (int k = 0; k < 3; ++k) v *= ipow(x[k], k == dir ? e - 1 : mono[m][k]);
        return v;
    }
    void eval(const double *xd, double *phi, double *grad /*[n][3]*/) const {
        const LD x[3] = {xd[0], xd[1], xd[2]};
        for (int k = 0; k < n; ++k) {
            LD v = 0, g[3] = {0, 0, 0};
            for (int m = 0; m < n; ++m) {
                LD c = coef[m * n + k];
                if (c == 0.0L) continue;
                v += c * mono_val(m, x);
                for (int dd = 0; dd < dim; ++dd) g[dd] += c * mono_der(m, dd, x);
            }
            if (phi) phi[k] = (double)v;
            if (grad)
                for (int dd = 0; dd < 3; ++dd) grad[k * 3 + dd] = (double)g[dd];
        }
    }
};

struct Rule {
    std::vector<double> uvwq;  // [g][4] as gmsh's parametric coords + weight
    int n = 0;
};
static Rule get_rule(int dim, int degree) {
    const double *t = nullptr;
    int n = 0;
#define PICK(D, NAME)    \
    if (degree == D) {   \
        t = NAME;        \
        n = NAME##_n;    \
    }
    if (dim == 1) { PICK(2, kLine2) PICK(4, kLine4) PICK(6, kLine6) PICK(8, kLine8) PICK(10, kLine10) }
    if (dim == 2) { PICK(2, kTri2) PICK(4, kTri4) PICK(6, kTri6) PICK(8, kTri8) PICK(10, kTri10) }
    if (dim == 3) { PICK(2, kTet2) PICK(4, kTet4) PICK(6, kTet6) PICK(8, kTet8) PICK(10, kTet10) }
#undef PICK
    if (!t) throw std::runtime_error("no quadrature rule");
    Rule r;
    r.n = n;
    r.uvwq.assign(t, t + 4 * n);
    return r;
}

// Jacobian of an element at a point (gmsh storage jac[u][x]), regularised
// for lower-dimensional elements; returns the gmsh determinant.
static double element_jacobian(const Basis &B, int edim, const std::vector<P3> &X, const double *grad,
                               double jac[3][3]) {
    for (int u = 0; u < 3; ++u)
        for (int x = 0; x < 3; ++x) jac[u][x] = 0.0;
    for (int k = 0; k < B.n; ++k)
        for (int u = 0; u < edim; ++u)
            for (int x = 0; x < 3; ++x) jac[u][x] += X[k][x] * grad[k * 3 + u];
    if (edim == 1) {
        double a[3] = {jac[0][0], jac[0][1], jac[0][2]}, b[3], c[3];
        double dJ = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if ((std::fabs(a[0]) >= std::fabs(a[1]) && std::fabs(a[0]) >= std::fabs(a[2])) ||
            (std::fabs(a[1]) >= std::fabs(a[0]) && std::fabs(a[1]) >= std::fabs(a[2]))) {
            b[0] = a[1]; b[1] = -a[0]; b[2] = 0.0;
        } else {
            b[0] = 0.0; b[1] = a[2]; b[2] = -a[1];
        }
        la::normalize(b, 3);
        la::cross(a, b, c);
        la::normalize(c, 3);
        for (int x = 0; x < 3; ++x) { jac[1][x] = b[x]; jac[2][x] = c[x]; }
        return dJ;
    }
    if (edim == 2) {
        double c[3];
        la::cross(jac[0], jac[1], c);
        double dJ = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        la::normalize(c, 3);
        for (int x = 0; x < 3; ++x) jac[2][x] = c[x];
        return dJ;
    }
    return jac[0][0] * jac[1][1] * jac[2][2] + jac[0][2] * jac[1][0] * jac[2][1] +
           jac[0][1] * jac[1][2] * jac[2][0] - jac[0][2] * jac[1][1] * jac[2][0] -
           jac[0][0] * jac[1][2] * jac[2][1] - jac[0][1] * jac[1][0] * jac[2][2];
}

// ---------------------------------------------------------------------------
// Model (what gmsh holds after gmsh::open) and configuration
// ---------------------------------------------------------------------------
struct Group {
    int dim, tag;
    std::vector<int> nodes;  // sorted
};
struct Model {
    int dim = 0, order = 0, np = 0;
    std::vector<int> node_tag;   // [nn]
    std::vector<double> xyz;     // [nn][3]
    std::vector<int> index;      // tag -> row
    std::vector<int> elTags, elNodeTags;
    std::vector<Group> groups;
    const double *getNode(int tag) const { return &xyz[index[tag] * 3]; }
};
struct Config {
    double timeStep = 0;
    int numThreads = 0;
    std::vector<double> v0 = {0, 0, 0};
    double rho0 = 1, c0 = 1;
    std::vector<std::vector<double>> sources;  // pole,x,y,z,size,amp,freq,phase,duration
    std::map<int, std::pair<std::string, double>> physBCs;
};

// ---------------------------------------------------------------------------
// Mesh (src/Mesh.cpp restated)
// ---------------------------------------------------------------------------
class OMesh {
public:
    OMesh(const Model &model, const Config &config);

    // accessors with the reference's index formulas (include/Mesh.h:31-108)
    int &elNodeTag(int el, int n = 0) { return m_elNodeTags[el * m_elNumNodes + n]; }
    double &elJacobian(int el, int g = 0, int x = 0, int u = 0) { return m_elJacobians[el * m_elNumIntPts * 9 + g * 9 + u * 3 + x]; }
    double &elJacobianDet(int el, int g = 0) { return m_elJacobianDets[el * m_elNumIntPts + g]; }
    double &elWeight(int g) { return m_elIntParamCoords[g * 4 + 3]; }
    double &elBasisFct(int g, int i = 0) { return m_elBasisFcts[g * m_elNumNodes + i]; }
    double &elUGradBasisFct(int g, int i = 0, int u = 0) { return m_elUGradBasisFcts[g * m_elNumNodes * 3 + i * 3 + u]; }
    double &elGradBasisFct(int el, int g = 0, int i = 0, int x = 0) {
        return m_elGradBasisFcts[(size_t)el * m_elNumIntPts * m_elNumNodes * 3 + g * m_elNumNodes * 3 + i * 3 + x];
    }
    int &elFNodeTag(int el, int f = 0, int i = 0) { return m_elFNodeTags[el * m_fNumPerEl * m_fNumNodes + f * m_fNumNodes + i]; }
    int &fNodeTag(int f, int i = 0) { return m_fNodeTags[f * m_fNumNodes + i]; }
    double &fJacobian(int f, int g = 0, int x = 0, int u = 0) { return m_fJacobians[f * m_fNumIntPts * 9 + g * 9 + u * 3 + x]; }
    double &fJacobianDet(int f, int g = 0) { return m_fJacobianDets[f * m_fNumIntPts + g]; }
    double &fUGradBasisFct(int g, int i = 0, int u = 0) { return m_fUGradBasisFcts[g * m_fNumNodes * 3 + i * 3 + u]; }
    double &fGradBasisFct(int f, int g = 0, int i = 0, int x = 0) {
        return m_fGradBasisFcts[(size_t)f * m_fNumIntPts * m_fNumNodes * 3 + g * m_fNumNodes * 3 + i * 3 + x];
    }
    double &fWeight(int g) { return m_fIntParamCoords[g * 4 + 3]; }
    double &fBasisFct(int g, int i = 0) { return m_fBasisFcts[g * m_fNumNodes + i]; }
    double &fNormal(int f, int g = 0, int x = 0) { return m_fNormals[f * 3 * m_fNumIntPts + g * 3 + x]; }
    int &elFId(int el, int f = 0) { return m_elFIds[el * m_fNumPerEl + f]; }
    int &fNbrElId(int f, int el = 0) { return m_fNbrElIds[f][el]; }
    int &fNToElNId(int f, int nf = 0, int el = 0) { return m_fNToElNIds[f][nf * m_fNbrElIds[f].size() + el]; }
    int &elFOrientation(int el, int f) { return m_elFOrientation[el * m_fNumPerEl + f]; }
    double &elMassMatrix(int el, int i = 0, int j = 0) {
        return m_elMassMatrices[(size_t)el * m_elNumNodes * m_elNumNodes + i * m_elNumNodes + j];
    }
    double &fFlux(int f, int n = 0) { return m_fFlux[f * m_fNumNodes + n]; }
    int getNumNodes() { return (int)m_elNodeTags.size(); }
    int getElNumNodes() { return m_elNumNodes; }
    int getElNum() { return m_elNum; }

    void getElMassMatrix(int el, bool inverse, double *elMassMatrix);
    void precomputeMassMatrix();
    void precomputeFlux(std::vector<double> &u, std::vector<std::vector<double>> &Flux, int eq);
    void getElFlux(int el, double *F);
    void getElStiffVector(int el, std::vector<std::vector<double>> &Flux, std::vector<double> &u, double *out);
    void updateFlux(std::vector<std::vector<double>> &u, std::vector<std::vector<std::vector<double>>> &Flux,
                    std::vector<double> &v0, double c0, double rho0);

    const Model &model;
    Config config;
    bool dedupFaceLoop = false;  // variant: the face loop once instead of once per outer thread
    // Option outside the reference: jump sign +1 on every interior face
    // (fc replaced per face by the first neighbour's orientation).
    bool upwind = false;
    std::vector<int> fcFace;  // per-face coefficient used in precomputeFlux

    int fc = 1;
    int m_Dim = 3;
    int m_elDim, m_elOrder, m_elNumNodes, m_elNumIntPts, m_elNum;
    std::vector<int> m_elTags, m_elNodeTags;
    std::vector<double> m_elJacobians, m_elJacobianDets, m_elIntParamCoords, m_elBasisFcts, m_elUGradBasisFcts,
        m_elGradBasisFcts;
    std::vector<int> m_elFIds, m_elFNodeTags, m_elFOrientation;
    int m_fDim, m_fNumNodes, m_fNumPerEl, m_fNum, m_fNumIntPts;
    std::vector<int> m_fNodeTags;
    std::vector<double> m_fJacobians, m_fJacobianDets, m_fIntParamCoords, m_fBasisFcts, m_fUGradBasisFcts,
        m_fGradBasisFcts, m_fNormals;
    std::vector<std::vector<int>> m_fNbrElIds, m_fNToElNIds;
    std::vector<double> m_elMassMatrices, m_fFlux;
    std::vector<bool> m_fIsBoundary;
    std::vector<int> m_fBC;
    std::vector<std::vector<double>> RKR;
    std::vector<std::vector<double>> uGhost;
    std::vector<std::vector<std::vector<double>>> FluxGhost;
};

struct VecHash {
    size_t operator()(const std::vector<int> &v) const {
        size_t h = 0xcbf29ce484222325ull;
        for (int x : v) { h ^= (size_t)(unsigned)x; h *= 0x100000001b3ull; }
        return h;
    }
};

OMesh::OMesh(const Model &mdl, const Config &cfg) : model(mdl), config(cfg) {
    // ---- Elements (Mesh.cpp:25-78)
    m_elDim = mdl.dim;
    m_elOrder = mdl.order;
    m_elNumNodes = mdl.np;
    m_elTags = mdl.elTags;
    m_elNodeTags = mdl.elNodeTags;
    m_elNum = (int)m_elTags.size();
    Basis eb;
    eb.build(m_elDim, m_elOrder);
    Rule er = get_rule(m_elDim, 2 * m_elOrder);
    m_elNumIntPts = er.n;
    m_elIntParamCoords = er.uvwq;
    m_elBasisFcts.resize(m_elNumIntPts * m_elNumNodes);
    m_elUGradBasisFcts.resize(m_elNumIntPts * m_elNumNodes * 3);
    for (int g = 0; g < m_elNumIntPts; ++g)
        eb.eval(&er.uvwq[g * 4], &m_elBasisFcts[g * m_elNumNodes], &m_elUGradBasisFcts[g * m_elNumNodes * 3]);
    m_elJacobians.resize((size_t)m_elNum * m_elNumIntPts * 9);
    m_elJacobianDets.resize((size_t)m_elNum * m_elNumIntPts);
    {
        std::vector<P3> X(m_elNumNodes);
        for (int el = 0; el < m_elNum; ++el) {
            for (int k = 0; k < m_elNumNodes; ++k) {
                const double *x = mdl.getNode(elNodeTag(el, k));
                X[k] = {x[0], x[1], x[2]};
            }
            for (int g = 0; g < m_elNumIntPts; ++g) {
                double jac[3][3];
                double dJ = element_jacobian(eb, m_elDim, X, &m_elUGradBasisFcts[g * m_elNumNodes * 3], jac);
                for (int u = 0; u < 3; ++u)
                    for (int x = 0; x < 3; ++x) elJacobian(el, g, x, u) = jac[u][x];
                elJacobianDet(el, g) = dJ;
            }
        }
    }
    std::vector<double> jacobian(m_elDim * m_elDim);
    m_elGradBasisFcts.assign((size_t)m_elNum * m_elNumNodes * m_elNumIntPts * 3, 0.0);
    for (int el = 0; el < m_elNum; ++el)
        for (int g = 0; g < m_elNumIntPts; ++g)
            for (int f = 0; f < m_elNumNodes; ++f) {
                for (int i = 0; i < m_elDim; ++i)
                    for (int j = 0; j < m_elDim; ++j) jacobian[i * m_elDim + j] = elJacobian(el, g, i, j);
                std::copy(&elUGradBasisFct(g, f), &elUGradBasisFct(g, f) + m_elDim, &elGradBasisFct(el, g, f));
                la::solve(jacobian.data(), &elGradBasisFct(el, g, f), m_elDim);
            }

    // ---- Faces (Mesh.cpp:92-159)
    m_fDim = m_elDim - 1;
    m_fNumNodes = m_fDim == 1 ? 1 + m_elOrder : (m_elOrder + 1) * (m_elOrder + 2) / 2;
    m_fNumPerEl = m_elDim + 1;
    // element face nodes in gmsh order: locate each face lattice point among
    // the element's reference nodes
    Basis fb;
    fb.build(m_fDim, m_elOrder);
    std::vector<std::vector<int>> faceLocal(m_fNumPerEl, std::vector<int>(m_fNumNodes));
    for (int lf = 0; lf < m_fNumPerEl; ++lf) {
        P3 v[3];
        for (int k = 0; k < m_elDim; ++k) {
            int vid = m_elDim == 2 ? kTriEdge[lf][k] : kTetFace[lf][k];
            v[k] = eb.nodes[vid];
        }
        for (int k = 0; k < m_fNumNodes; ++k) {
            P3 q;
            const P3 &r = fb.nodes[k];
            if (m_fDim == 1) {
                double t = 0.5 * (r[0] + 1.0);
                for (int x = 0; x < 3; ++x) q[x] = v[0][x] + t * (v[1][x] - v[0][x]);
            } else {
                for (int x = 0; x < 3; ++x) q[x] = v[0][x] + r[0] * (v[1][x] - v[0][x]) + r[1] * (v[2][x] - v[0][x]);
            }
            int found = -1;
            for (int i = 0; i < m_elNumNodes; ++i)
                if (std::fabs(eb.nodes[i][0] - q[0]) + std::fabs(eb.nodes[i][1] - q[1]) +
                        std::fabs(eb.nodes[i][2] - q[2]) < 1e-12)
                    found = i;
            if (found < 0) throw std::runtime_error("face node not found on the reference element");
            faceLocal[lf][k] = found;
        }
    }
    m_elFNodeTags.resize((size_t)m_elNum * m_fNumPerEl * m_fNumNodes);
    for (int el = 0; el < m_elNum; ++el)
        for (int lf = 0; lf < m_fNumPerEl; ++lf)
            for (int k = 0; k < m_fNumNodes; ++k) elFNodeTag(el, lf, k) = elNodeTag(el, faceLocal[lf][k]);
    // unique faces, first occurrence kept (getUniqueFaceNodeTags), and the
    // element-face connectivity (Mesh.cpp:235-246)
    std::unordered_map<std::vector<int>, int, VecHash> seen;
    std::vector<int> key(m_fNumNodes);
    for (int el = 0; el < m_elNum; ++el)
        for (int elF = 0; elF < m_fNumPerEl; ++elF) {
            for (int k = 0; k < m_fNumNodes; ++k) key[k] = elFNodeTag(el, elF, k);
            std::sort(key.begin(), key.end());
            auto it = seen.find(key);
            int f;
            if (it == seen.end()) {
                f = (int)m_fNbrElIds.size();
                seen.emplace(key, f);
                m_fNbrElIds.push_back({});
                for (int k = 0; k < m_fNumNodes; ++k) m_fNodeTags.push_back(elFNodeTag(el, elF, k));
            } else {
                f = it->second;
            }
            m_elFIds.push_back(f);
            m_fNbrElIds[f].push_back(el);
        }
    m_fNum = (int)m_fNbrElIds.size();
    // face element data
    Rule fr = get_rule(m_fDim, 2 * m_elOrder);
    m_fNumIntPts = fr.n;
    m_fIntParamCoords = fr.uvwq;
    m_fBasisFcts.resize(m_fNumIntPts * m_fNumNodes);
    m_fUGradBasisFcts.resize(m_fNumIntPts * m_fNumNodes * 3);
    for (int g = 0; g < m_fNumIntPts; ++g)
        fb.eval(&fr.uvwq[g * 4], &m_fBasisFcts[g * m_fNumNodes], &m_fUGradBasisFcts[g * m_fNumNodes * 3]);
    m_fJacobians.resize((size_t)m_fNum * m_fNumIntPts * 9);
    m_fJacobianDets.resize((size_t)m_fNum * m_fNumIntPts);
    {
        std::vector<P3> X(m_fNumNodes);
        for (int f = 0; f < m_fNum; ++f) {
            for (int k = 0; k < m_fNumNodes; ++k) {
                const double *x = mdl.getNode(fNodeTag(f, k));
                X[k] = {x[0], x[1], x[2]};
            }
            for (int g = 0; g < m_fNumIntPts; ++g) {
                double jac[3][3];
                double dJ = element_jacobian(fb, m_fDim, X, &m_fUGradBasisFcts[g * m_fNumNodes * 3], jac);
                for (int u = 0; u < 3; ++u)
                    for (int x = 0; x < 3; ++x) fJacobian(f, g, x, u) = jac[u][x];
                fJacobianDet(f, g) = dJ;
            }
        }
    }
    m_fGradBasisFcts.assign((size_t)m_fNum * m_fNumNodes * m_fNumIntPts * 3, 0.0);
    for (int f = 0; f < m_fNum; ++f)
        for (int g = 0; g < m_fNumIntPts; ++g)
            for (int n = 0; n < m_fNumNodes; ++n) {
                for (int i = 0; i < m_elDim; ++i)
                    for (int j = 0; j < m_elDim; ++j) jacobian[i * m_elDim + j] = fJacobian(f, g, i, j);
                std::copy(&fUGradBasisFct(g, n), &fUGradBasisFct(g, n) + m_elDim, &fGradBasisFct(f, g, n));
                la::solve(jacobian.data(), &fGradBasisFct(f, g, n), m_elDim);
            }
    // normals (Mesh.cpp:164-194)
    std::vector<double> normal(m_Dim);
    for (int f = 0; f < m_fNum; ++f)
        for (int g = 0; g < m_fNumIntPts; ++g) {
            if (m_fDim == 1) {
                double normalPlane[3] = {0, 0, -1};
                la::cross(&fGradBasisFct(f, g, 0), normalPlane, normal.data());
                if (la::dot(&fGradBasisFct(f, g), &fGradBasisFct(f, 0), m_Dim) < 0)
                    for (int x = 0; x < m_Dim; ++x) normal[x] = -normal[x];
            } else {
                la::cross(&fGradBasisFct(f, g, 0), &fGradBasisFct(f, g, 1), normal.data());
                if (g != 0 && la::dot(&fNormal(f, 0), normal.data(), m_Dim) < 0)
                    for (int x = 0; x < m_Dim; ++x) normal[x] = -normal[x];
            }
            la::normalize(normal.data(), m_Dim);
            m_fNormals.insert(m_fNormals.end(), normal.begin(), normal.end());
        }
    if (m_elDim == 3 && m_elOrder != 1) fc = -1;

    // ---- face node -> element node (Mesh.cpp:253-263)
    m_fNToElNIds.resize(m_fNum);
    for (int f = 0; f < m_fNum; ++f)
        for (int nf = 0; nf < m_fNumNodes; ++nf)
            for (int el : m_fNbrElIds[f])
                for (int nel = 0; nel < m_elNumNodes; ++nel)
                    if (fNodeTag(f, nf) == elNodeTag(el, nel)) m_fNToElNIds[f].push_back(nel);
    // ---- orientation (Mesh.cpp:278-294), barycentres of the primary nodes
    for (int el = 0; el < m_elNum; ++el) {
        double bc[3] = {0, 0, 0};
        for (int v = 0; v <= m_elDim; ++v) {
            const double *x = mdl.getNode(elNodeTag(el, v));
            for (int k = 0; k < 3; ++k) bc[k] += x[k];
        }
        for (int k = 0; k < 3; ++k) bc[k] /= (m_elDim + 1);
        for (int f = 0; f < m_fNumPerEl; ++f) {
            double dotProduct = 0.0;
            const double *fNodeCoord = mdl.getNode(elFNodeTag(el, f));
            for (int x = 0; x < m_Dim; ++x) dotProduct += (fNodeCoord[x] - bc[x]) * fNormal(elFId(el, f), 0, x);
            m_elFOrientation.push_back(dotProduct >= 0 ? 1 : -1);
        }
    }
    // ---- neighbour reordering (Mesh.cpp:301-314); its guard compares the
    // number of faces with 2
    int elf = 0;
    for (int f = 0; f < m_fNum; ++f) {
        for (int lf = 0; lf < m_fNumPerEl; ++lf)
            if (elFId(fNbrElId(f, 0), lf) == f) elf = lf;
        if (m_fNbrElIds.size() == 2 && m_fNbrElIds[f].size() == 2) {
            if (elFOrientation(fNbrElId(f, 0), elf) <= 0) {
                std::swap(m_fNbrElIds[f][0], m_fNbrElIds[f][1]);
                for (int nf = 0; nf < m_fNumNodes; ++nf) std::swap(fNToElNId(f, nf, 0), fNToElNId(f, nf, 1));
            }
        }
    }
    // ---- boundary faces (Mesh.cpp:336-353)
    for (int f = 0; f < m_fNum; ++f) {
        if (m_fNbrElIds[f].size() < 2) {
            m_fIsBoundary.push_back(true);
            for (int lf = 0; lf < m_fNumPerEl; ++lf)
                if (elFId(fNbrElId(f, 0), lf) == f) {
                    for (int g = 0; g < m_fNumIntPts; ++g)
                        for (int x = 0; x < 3; ++x) fNormal(f, g, x) *= elFOrientation(fNbrElId(f, 0), lf);
                    elFOrientation(fNbrElId(f, 0), lf) = 1;
                }
        } else {
            m_fIsBoundary.push_back(false);
        }
    }
    // ---- boundary conditions (Mesh.cpp:364-384)
    m_fBC.resize(m_fNum);
    for (auto const &physBC : config.physBCs) {
        const Group *grp = nullptr;
        for (auto &g : mdl.groups)
            if (g.dim == m_fDim && g.tag == physBC.first) grp = &g;
        static const std::vector<int> none;
        const std::vector<int> &nodeTags = grp ? grp->nodes : none;
        int val = physBC.second.first == "Reflecting" ? 1 : 0;
        for (int f = 0; f < m_fNum; ++f)
            if (m_fIsBoundary[f] && std::binary_search(nodeTags.begin(), nodeTags.end(), fNodeTag(f))) m_fBC[f] = val;
    }
    // ---- absorbing matrix (Mesh.cpp:391-418)
    RKR.resize((size_t)m_fNum * m_fNumIntPts);
    const double c0 = config.c0, rho0 = config.rho0;
    for (int f = 0; f < m_fNum; ++f) {
        if (m_fBC[f] != 0) continue;
        for (int g = 0; g < m_fNumIntPts; ++g) {
            int i = f * m_fNumIntPts + g;
            double n0 = fNormal(f, g, 0), n1 = fNormal(f, g, 1), n2 = fNormal(f, g, 2);
            RKR[i] = {0.25 * c0, 0.25 * c0 * c0 * rho0 * n0, 0.25 * c0 * c0 * rho0 * n1, 0.25 * c0 * c0 * rho0 * n2,
                      0.25 * n0 / rho0, 0.25 * c0 * n0 * n0, 0.25 * c0 * n0 * n1, 0.25 * c0 * n0 * n2,
                      0.25 * n1 / rho0, 0.25 * c0 * n1 * n0, 0.25 * c0 * n1 * n1, 0.25 * c0 * n1 * n2,
                      0.25 * n2 / rho0, 0.25 * c0 * n2 * n0, 0.25 * c0 * n2 * n1, 0.25 * c0 * n2 * n2};
        }
    }
    fcFace.assign(m_fNum, fc);
    m_fFlux.resize((size_t)m_fNum * m_fNumNodes);
    uGhost = std::vector<std::vector<double>>(4, std::vector<double>((size_t)m_fNum * m_fNumIntPts));
    FluxGhost = std::vector<std::vector<std::vector<double>>>(
        4, std::vector<std::vector<double>>((size_t)m_fNum * m_fNumIntPts, std::vector<double>(3)));
}

void OMesh::precomputeMassMatrix() {
    m_elMassMatrices.resize((size_t)m_elNum * m_elNumNodes * m_elNumNodes);
    for (int el = 0; el < m_elNum; ++el) getElMassMatrix(el, true, &elMassMatrix(el));
}

void OMesh::getElMassMatrix(const int el, const bool inverse, double *M) {
    for (int i = 0; i < m_elNumNodes; ++i)
        for (int j = 0; j < m_elNumNodes; ++j) {
            M[i * m_elNumNodes + j] = 0.0;
            for (int g = 0; g < m_elNumIntPts; g++)
                M[i * m_elNumNodes + j] += elBasisFct(g, i) * elBasisFct(g, j) * elWeight(g) * elJacobianDet(el, g);
        }
    // (the reference also builds a JacobiSVD here and discards it)
    if (inverse) la::inverse(M, m_elNumNodes);
}

void OMesh::getElStiffVector(const int el, std::vector<std::vector<double>> &Flux, std::vector<double> &u,
                             double *elStiffVector) {
    (void)u;
    int jId;
    for (int i = 0; i < m_elNumNodes; ++i) {
        elStiffVector[i] = 0.0;
        for (int j = 0; j < m_elNumNodes; ++j) {
            jId = el * m_elNumNodes + j;
            for (int g = 0; g < m_elNumIntPts; g++)
                elStiffVector[i] += la::dot(Flux[jId].data(), &elGradBasisFct(el, g, i), m_Dim) * elBasisFct(g, j) *
                                    elWeight(g) * elJacobianDet(el, g);
        }
    }
}

void OMesh::precomputeFlux(std::vector<double> &u, std::vector<std::vector<double>> &Flux, int eq) {
    auto body = [&](int f, std::vector<double> &FIntPts, std::vector<double> &Fnum) {
        int elUp, elDn;
        std::fill(FIntPts.begin(), FIntPts.end(), 0);
        if (m_fIsBoundary[f]) {
            for (int g = 0; g < m_fNumIntPts; ++g) FIntPts[g] = FluxGhost[eq][f * m_fNumIntPts + g][0];
        } else {
            for (int i = 0; i < m_fNumNodes; ++i) {
                elUp = fNbrElId(f, 0) * m_elNumNodes + fNToElNId(f, i, 0);
                elDn = fNbrElId(f, 1) * m_elNumNodes + fNToElNId(f, i, 1);
                for (int g = 0; g < m_fNumIntPts; ++g) {
                    for (int x = 0; x < m_Dim; ++x)
                        Fnum[x] = 0.5 * ((Flux[elUp][x] + Flux[elDn][x]) +
                                         fcFace[f] * config.c0 * fNormal(f, g, x) * (u[elUp] - u[elDn]));
                    FIntPts[g] += la::dot(&fNormal(f, g), Fnum.data(), m_Dim) * fBasisFct(g, i);
                }
            }
        }
        for (int n = 0; n < m_fNumNodes; ++n) {
            fFlux(f, n) = 0;
            for (int g = 0; g < m_fNumIntPts; ++g)
                fFlux(f, n) += fWeight(g) * fBasisFct(g, n) * FIntPts[g] * fJacobianDet(f, g);
        }
    };
    if (dedupFaceLoop) {
#pragma omp parallel num_threads(config.numThreads)
        {
            std::vector<double> FIntPts(m_fNumIntPts, 0), Fnum(m_Dim, 0);
#pragma omp for schedule(static)
            for (int f = 0; f < m_fNum; ++f) body(f, FIntPts, Fnum);
        }
        return;
    }
#pragma omp parallel num_threads(config.numThreads)
    {
        std::vector<double> FIntPts(m_fNumIntPts, 0);
        std::vector<double> Fnum(m_Dim, 0);
#pragma omp parallel for schedule(static)
        for (int f = 0; f < m_fNum; ++f) body(f, FIntPts, Fnum);
    }
}

void OMesh::getElFlux(const int el, double *F) {
    int i;
    std::fill(F, F + m_elNumNodes, 0);
    for (int f = 0; f < m_fNumPerEl; ++f) {
        el == fNbrElId(elFId(el, f), 0) ? i = 0 : i = 1;
        for (int nf = 0; nf < m_fNumNodes; ++nf)
            F[fNToElNId(elFId(el, f), nf, i)] += elFOrientation(el, f) * fFlux(elFId(el, f), nf);
    }
}

void OMesh::updateFlux(std::vector<std::vector<double>> &u, std::vector<std::vector<std::vector<double>>> &Flux,
                       std::vector<double> &v0, double c0, double rho0) {
    for (int el = 0; el < m_elNum; ++el) {
        for (int n = 0; n < m_elNumNodes; ++n) {
            int i = el * m_elNumNodes + n;
            Flux[0][i] = {v0[0] * u[0][i] + rho0 * c0 * c0 * u[1][i], v0[1] * u[0][i] + rho0 * c0 * c0 * u[2][i],
                          v0[2] * u[0][i] + rho0 * c0 * c0 * u[3][i]};
            Flux[1][i] = {v0[0] * u[1][i] + u[0][i] / rho0, v0[1] * u[1][i], v0[2] * u[1][i]};
            Flux[2][i] = {v0[0] * u[2][i], v0[1] * u[2][i] + u[0][i] / rho0, v0[2] * u[2][i]};
            Flux[3][i] = {v0[0] * u[3][i], v0[1] * u[3][i], v0[2] * u[3][i] + u[0][i] / rho0};
        }
        for (int f = 0; f < m_fNumPerEl; ++f) {
            int fId = elFId(el, f);
            if (!m_fIsBoundary[fId]) continue;
            for (int g = 0; g < m_fNumIntPts; ++g) {
                int gId = fId * m_fNumIntPts + g;
                uGhost[0][gId] = uGhost[1][gId] = uGhost[2][gId] = uGhost[3][gId] = 0;
                for (int n = 0; n < m_fNumNodes; ++n) {
                    int nId = el * m_elNumNodes + fNToElNId(fId, n, 0);
                    for (int q = 0; q < 4; ++q) uGhost[q][gId] += u[q][nId] * fBasisFct(g, n);
                }
                if (m_fBC[fId] == 1) {
                    double dot = fNormal(fId, g, 0) * uGhost[1][gId] + fNormal(fId, g, 1) * uGhost[2][gId] +
                                 fNormal(fId, g, 2) * uGhost[3][gId];
                    uGhost[1][gId] -= dot * fNormal(fId, g, 0);
                    uGhost[2][gId] -= dot * fNormal(fId, g, 1);
                    uGhost[3][gId] -= dot * fNormal(fId, g, 2);
                    FluxGhost[0][gId] = {v0[0] * uGhost[0][gId] + rho0 * c0 * c0 * uGhost[1][gId],
                                         v0[1] * uGhost[0][gId] + rho0 * c0 * c0 * uGhost[2][gId],
                                         v0[2] * uGhost[0][gId] + rho0 * c0 * c0 * uGhost[3][gId]};
                    FluxGhost[1][gId] = {v0[0] * uGhost[1][gId] + uGhost[0][gId] / rho0, v0[1] * uGhost[1][gId],
                                         v0[2] * uGhost[1][gId]};
                    FluxGhost[2][gId] = {v0[0] * uGhost[2][gId], v0[1] * uGhost[2][gId] + uGhost[0][gId] / rho0,
                                         v0[2] * uGhost[2][gId]};
                    FluxGhost[3][gId] = {v0[0] * uGhost[3][gId], v0[1] * uGhost[3][gId],
                                         v0[2] * uGhost[3][gId] + uGhost[0][gId] / rho0};
                    for (int eq = 0; eq < 4; ++eq)
                        FluxGhost[eq][gId][0] = la::dot(&fNormal(fId, g), &FluxGhost[eq][gId][0], m_Dim);
                } else {
                    for (int eq = 0; eq < 4; ++eq)
                        FluxGhost[eq][gId][0] = RKR[gId][eq * 4 + 0] * uGhost[0][gId] + RKR[gId][eq * 4 + 1] * uGhost[1][gId] +
                                                RKR[gId][eq * 4 + 2] * uGhost[2][gId] + RKR[gId][eq * 4 + 3] * uGhost[3][gId];
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Solver (src/solver.cpp restated)
// ---------------------------------------------------------------------------
struct Solver {
    OMesh *mesh = nullptr;
    Config config;
    int elNumNodes = 0, numNodes = 0;
    std::vector<double> elFlux, elStiffvector;
    std::vector<std::vector<std::vector<double>>> Flux;
    std::vector<std::vector<double>> u, k1, k2, k3, k4;
    std::vector<std::vector<int>> srcIndices;
    // Per-node weights of Gaussian-in-space sources (type 1, not a reference
    // source type: nodes within 3 sigma, weight exp(-r^2 / (2 sigma^2)),
    // sigma = the size field); reference sources (type 0) have weight 1.
    std::vector<std::vector<double>> srcWeights;

    void numStep(std::vector<std::vector<double>> &uu, double beta) {
        for (int eq = 0; eq < 4; ++eq) {
            mesh->precomputeFlux(uu[eq], Flux[eq], eq);
#pragma omp parallel for schedule(static) firstprivate(elFlux, elStiffvector) num_threads(config.numThreads)
            for (int el = 0; el < mesh->getElNum(); ++el) {
                mesh->getElFlux(el, elFlux.data());
                mesh->getElStiffVector(el, Flux[eq], uu[eq], elStiffvector.data());
                la::minus(elStiffvector.data(), elFlux.data(), elNumNodes);
                la::linEq(&mesh->elMassMatrix(el), &elStiffvector[0], &uu[eq][el * elNumNodes], config.timeStep,
                          beta, elNumNodes);
            }
        }
    }

    void setup() {
        elNumNodes = mesh->getElNumNodes();
        numNodes = mesh->getNumNodes();
        elFlux.resize(elNumNodes);
        elStiffvector.resize(elNumNodes);
        Flux = std::vector<std::vector<std::vector<double>>>(
            4, std::vector<std::vector<double>>(numNodes, std::vector<double>(3)));
        mesh->precomputeMassMatrix();
        srcIndices.clear();
        srcWeights.clear();
        for (size_t i = 0; i < config.sources.size(); ++i) {
            std::vector<int> indice;
            std::vector<double> weight;
            const bool gaussian = config.sources[i][0] == 1.0;
            const double radius = gaussian ? 3.0 * config.sources[i][4] : config.sources[i][4];
            for (int n = 0; n < numNodes; n++) {
                const double *coord = mesh->model.getNode(mesh->m_elNodeTags[n]);
                const double r2 = std::pow(coord[0] - config.sources[i][1], 2) +
                                  std::pow(coord[1] - config.sources[i][2], 2) +
                                  std::pow(coord[2] - config.sources[i][3], 2);
                if (r2 < std::pow(radius, 2)) {
                    indice.push_back(n);
                    const double sg = config.sources[i][4];
                    weight.push_back(gaussian ? std::exp(-r2 / (2 * sg * sg)) : 1.0);
                }
            }
            srcIndices.push_back(indice);
            srcWeights.push_back(weight);
        }
        u.assign(4, std::vector<double>(numNodes, 0.0));
    }

    // Time integrator: 0 = "Runge-Kutta" (solver.cpp:171-292), 1 = "Euler1"
    // (solver.cpp:61-161).
    int method = 0;

    // One iteration of the time loop body (sources, then the integrator).
    void step(double t) {
        for (size_t src = 0; src < config.sources.size(); ++src) {
            double amp = config.sources[src][5], freq = config.sources[src][6];
            double phase = config.sources[src][7], duration = config.sources[src][8];
            if (t < duration)
                for (size_t n = 0; n < srcIndices[src].size(); ++n)
                    u[0][srcIndices[src][n]] = srcWeights[src][n] * (amp * std::sin(2 * M_PI * freq * t + phase));
        }
        if (method == 1) {
            // first-order Euler in place: solver.cpp:152-153 (numStep with beta = 1)
            mesh->updateFlux(u, Flux, config.v0, config.c0, config.rho0);
            numStep(u, 1);
            return;
        }
        k1 = k2 = k3 = k4 = u;
        mesh->updateFlux(k1, Flux, config.v0, config.c0, config.rho0);
        numStep(k1, 0);
        for (size_t eq = 0; eq < u.size(); ++eq) la::plusTimes(k2[eq].data(), k1[eq].data(), 0.5, numNodes);
        mesh->updateFlux(k2, Flux, config.v0, config.c0, config.rho0);
        numStep(k2, 0);
        for (size_t eq = 0; eq < u.size(); ++eq) la::plusTimes(k3[eq].data(), k2[eq].data(), 0.5, numNodes);
        mesh->updateFlux(k3, Flux, config.v0, config.c0, config.rho0);
        numStep(k3, 0);
        for (size_t eq = 0; eq < u.size(); ++eq) la::plusTimes(k4[eq].data(), k3[eq].data(), 1, numNodes);
        mesh->updateFlux(k4, Flux, config.v0, config.c0, config.rho0);
        numStep(k4, 0);
        for (size_t eq = 0; eq < u.size(); ++eq)
            for (int i = 0; i < numNodes; ++i) u[eq][i] += (k1[eq][i] + 2 * k2[eq][i] + 2 * k3[eq][i] + k4[eq][i]) / 6.0;
    }
};

struct Handle {
    Model model;
    OMesh *mesh = nullptr;
    Solver solver;
    std::string err;
    ~Handle() { delete mesh; }
};

}  // namespace oracle

using namespace oracle;

extern "C" {

// Mesh as read from a .msh file and the configuration values the path uses.
typedef struct oracle_input {
    int dim, order, np;
    int num_nodes;
    const int *node_tags;
    const double *xyz;
    int num_el;
    const int *el_tags;
    const int *el_nodes;
    int num_groups;
    const int *group_dim, *group_tag, *group_offsets, *group_nodes;
    double time_step;
    int num_threads;
    double v0[3];
    double rho0, c0;
    int num_sources;
    const double *sources;  // [n][9]
    int num_bcs;
    const int *bc_tags;
    const int *bc_reflecting;
    int upwind;  // 1: jump sign +1 on every interior face (not a reference mode)
} oracle_input;

void *oracle_create(const oracle_input *in, char *err, int errlen) {
    auto *h = new Handle();
    try {
        Model &m = h->model;
        m.dim = in->dim;
        m.order = in->order;
        m.np = in->np;
        m.node_tag.assign(in->node_tags, in->node_tags + in->num_nodes);
        m.xyz.assign(in->xyz, in->xyz + 3 * (size_t)in->num_nodes);
        int mx = 0;
        for (int t : m.node_tag) mx = std::max(mx, t);
        m.index.assign(mx + 1, -1);
        for (int i = 0; i < in->num_nodes; ++i) m.index[m.node_tag[i]] = i;
        m.elTags.assign(in->el_tags, in->el_tags + in->num_el);
        m.elNodeTags.assign(in->el_nodes, in->el_nodes + (size_t)in->num_el * in->np);
        for (int g = 0; g < in->num_groups; ++g) {
            Group gr;
            gr.dim = in->group_dim[g];
            gr.tag = in->group_tag[g];
            gr.nodes.assign(in->group_nodes + in->group_offsets[g], in->group_nodes + in->group_offsets[g + 1]);
            std::sort(gr.nodes.begin(), gr.nodes.end());
            m.groups.push_back(gr);
        }
        Config c;
        c.timeStep = in->time_step;
        // the reference's numThreads key: 1 is read as 0, the OpenMP default
        // team (configParser.cpp:57-58).  With a one-thread outer team the
        // nested face loop's inner `parallel for` would become the active
        // level and share the outer region's scratch vectors across threads;
        // the reference never reaches that state, and neither does the oracle.
        c.numThreads = in->num_threads == 1 ? 0 : in->num_threads;
        c.v0 = {in->v0[0], in->v0[1], in->v0[2]};
        c.rho0 = in->rho0;
        c.c0 = in->c0;
        for (int s = 0; s < in->num_sources; ++s) c.sources.emplace_back(in->sources + 9 * s, in->sources + 9 * s + 9);
        for (int b = 0; b < in->num_bcs; ++b)
            c.physBCs[in->bc_tags[b]] = std::make_pair(in->bc_reflecting[b] ? "Reflecting" : "Absorbing", 0.0);
        h->mesh = new OMesh(h->model, c);
        if (in->upwind) {
            OMesh &om = *h->mesh;
            om.upwind = true;
            for (int f = 0; f < om.m_fNum; ++f) {
                if (om.m_fNbrElIds[f].size() < 2) continue;
                int e0 = om.fNbrElId(f, 0);
                for (int lf = 0; lf < om.m_fNumPerEl; ++lf)
                    if (om.elFId(e0, lf) == f) om.fcFace[f] = om.elFOrientation(e0, lf);
            }
        }
        h->solver.mesh = h->mesh;
        h->solver.config = c;
        h->solver.setup();
    } catch (std::exception &e) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.what());
        delete h;
        return nullptr;
    }
    return h;
}

void oracle_destroy(void *p) { delete (Handle *)p; }

// Reference-element data as the oracle builds it for elements of the given
// dimension (1-3) and order: its node lattice (gmsh order), its Gauss(2p)
// rule, and the matrices that rule gives with its Lagrange basis
//   mass[i*n + j]          = sum_g w_g phi_i(g) phi_j(g)
//   stiff[(u*n + i)*n + j] = sum_g w_g dphi_i/du(g) phi_j(g)   (u < dim)
// and the basis at the rule points, phi[g*n + i] and grad[(g*n + i)*3 + u].
// Any output pointer may be null.  Returns n (nodes), *ng the rule's point
// count, or -1 when no rule exists.  Used by the tests that pin the
// restated basis and rules against exact rational integrals.
int oracle_reference_element(int dim, int order, double *nodes, double *mass, double *stiff, int *ng,
                             double *rule, double *phi_out, double *grad_out) {
    if (dim < 1 || dim > 3 || order < 1 || order > 5) return -1;
    try {
        Basis b;
        b.build(dim, order);
        Rule r = get_rule(dim, 2 * order);
        int n = b.n;
        if (ng) *ng = r.n;
        if (rule) std::copy(r.uvwq.begin(), r.uvwq.end(), rule);
        if (nodes)
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) nodes[i * 3 + k] = b.nodes[i][k];
        std::vector<double> phi((size_t)r.n * n), grad((size_t)r.n * n * 3);
        for (int g = 0; g < r.n; ++g) b.eval(&r.uvwq[g * 4], &phi[(size_t)g * n], &grad[(size_t)g * n * 3]);
        if (phi_out) std::copy(phi.begin(), phi.end(), phi_out);
        if (grad_out) std::copy(grad.begin(), grad.end(), grad_out);
        if (mass)
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    double s = 0;
                    for (int g = 0; g < r.n; ++g) s += r.uvwq[g * 4 + 3] * phi[g * n + i] * phi[g * n + j];
                    mass[i * n + j] = s;
                }
        if (stiff)
            for (int u = 0; u < dim; ++u)
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) {
                        double s = 0;
                        for (int g = 0; g < r.n; ++g)
                            s += r.uvwq[g * 4 + 3] * grad[(g * n + i) * 3 + u] * phi[g * n + j];
                        stiff[(u * n + i) * n + j] = s;
                    }
        return n;
    } catch (std::exception &) {
        return -1;
    }
}

// 0 = classical RK4 ("Runge-Kutta"), 1 = forward Euler ("Euler1").
int oracle_set_method(void *p, int method) {
    if (method != 0 && method != 1) return -1;
    ((Handle *)p)->solver.method = method;
    return 0;
}

int oracle_num_dofs(void *p) { return ((Handle *)p)->solver.numNodes; }

int oracle_set_state(void *p, const double *u) {
    auto *h = (Handle *)p;
    for (int q = 0; q < 4; ++q)
        std::copy(u + (size_t)q * h->solver.numNodes, u + (size_t)(q + 1) * h->solver.numNodes, h->solver.u[q].begin());
    return 0;
}

int oracle_get_state(void *p, double *u) {
    auto *h = (Handle *)p;
    for (int q = 0; q < 4; ++q) std::copy(h->solver.u[q].begin(), h->solver.u[q].end(), u + (size_t)q * h->solver.numNodes);
    return 0;
}

// nsteps iterations of the loop body starting at *t (t += dt accumulated);
// *seconds = wall time of the loop.  dedup: face loop once, not per thread.
int oracle_run(void *p, double *t, int nsteps, int dedup, double *seconds) {
    auto *h = (Handle *)p;
    h->mesh->dedupFaceLoop = dedup != 0;
    auto t0 = std::chrono::steady_clock::now();
    double tt = *t;
    for (int k = 0; k < nsteps; ++k) {
        h->solver.step(tt);
        tt += h->solver.config.timeStep;
    }
    auto t1 = std::chrono::steady_clock::now();
    *t = tt;
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

// Reference loop of solver.cpp:216-217: runs while t <= time_end; returns the
// number of steps taken.
int oracle_run_until(void *p, double t_start, double time_end, double *seconds) {
    auto *h = (Handle *)p;
    auto t0 = std::chrono::steady_clock::now();
    int steps = 0;
    for (double t = t_start; t <= time_end; t += h->solver.config.timeStep) {
        h->solver.step(t);
        ++steps;
    }
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return steps;
}

// Precompute arrays for comparison with the product's mesh layer (values at
// the first quadrature point).
typedef struct oracle_mesh_view {
    int fc, num_el, f_num, nf, nfp, np, n_el_qp, n_f_qp;
    const int *el_f_ids;
    const int *el_f_orientation;
    const int *f_node_tags;
    const int *f_bc;
    const double *el_jac_dets;  // [num_el][n_el_qp]
    const double *f_jac_dets;   // [f_num][n_f_qp]
    const double *f_normals;    // [f_num][n_f_qp][3]
} oracle_mesh_view;

int oracle_mesh(void *p, oracle_mesh_view *v) {
    auto *h = (Handle *)p;
    OMesh &m = *h->mesh;
    v->fc = m.fc;
    v->num_el = m.m_elNum;
    v->f_num = m.m_fNum;
    v->nf = m.m_fNumPerEl;
    v->nfp = m.m_fNumNodes;
    v->np = m.m_elNumNodes;
    v->n_el_qp = m.m_elNumIntPts;
    v->n_f_qp = m.m_fNumIntPts;
    v->el_f_ids = m.m_elFIds.data();
    v->el_f_orientation = m.m_elFOrientation.data();
    v->f_node_tags = m.m_fNodeTags.data();
    v->f_bc = m.m_fBC.data();
    v->el_jac_dets = m.m_elJacobianDets.data();
    v->f_jac_dets = m.m_fJacobianDets.data();
    v->f_normals = m.m_fNormals.data();
    return 0;
}

// Neighbours and face-node map, flattened to [F][2] and [F][nfp][2] (-1 fill).
int oracle_face_maps(void *p, int *nbr, int *fn2en) {
    auto *h = (Handle *)p;
    OMesh &m = *h->mesh;
    for (int f = 0; f < m.m_fNum; ++f) {
        size_t cnt = m.m_fNbrElIds[f].size();
        for (int s = 0; s < 2; ++s) nbr[f * 2 + s] = s < (int)cnt ? m.m_fNbrElIds[f][s] : -1;
        for (int k = 0; k < m.m_fNumNodes; ++k)
            for (int s = 0; s < 2; ++s)
                fn2en[((size_t)f * m.m_fNumNodes + k) * 2 + s] = s < (int)cnt ? m.fNToElNId(f, k, s) : -1;
    }
    return 0;
}

// One right-hand side evaluation dt*M^-1(S-F) of a given state (no RK).
int oracle_rhs(void *p, const double *uin, double *out) {
    auto *h = (Handle *)p;
    Solver &s = h->solver;
    std::vector<std::vector<double>> w(4, std::vector<double>(s.numNodes));
    for (int q = 0; q < 4; ++q) std::copy(uin + (size_t)q * s.numNodes, uin + (size_t)(q + 1) * s.numNodes, w[q].begin());
    s.mesh->updateFlux(w, s.Flux, s.config.v0, s.config.c0, s.config.rho0);
    s.numStep(w, 0);
    for (int q = 0; q < 4; ++q) std::copy(w[q].begin(), w[q].end(), out + (size_t)q * s.numNodes);
    return 0;
}

}  // extern "C"
