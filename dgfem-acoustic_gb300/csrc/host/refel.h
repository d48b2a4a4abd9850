// Reference simplex elements for the nodal DG operators.
//
// Node ordering follows the gmsh convention that the reference reads through
// gmsh::model::mesh::getElementsByType / getElementFaceNodes (Mesh.cpp:29,110):
// vertices, then edge nodes edge by edge in the edge's direction, then face
// interior nodes, then volume interior nodes (recursively, as a lower order
// simplex).  Triangle edges are {0,1},{1,2},{2,0}; tetrahedron edges are
// {0,1},{1,2},{2,0},{3,0},{3,2},{3,1} and faces {0,2,1},{0,1,3},{0,3,2},{3,1,2}.
//
// Reference coordinates are gmsh's: line u in [-1,1]; triangle (0,0),(1,0),(0,1);
// tetrahedron (0,0,0),(1,0,0),(0,1,0),(0,0,1).
//
// The operators are built from the orthonormal Koornwinder-Dubiner basis and
// its Vandermonde matrix (Hesthaven & Warburton, "Nodal Discontinuous Galerkin
// Methods", 2008, ch. 6 and 10), so no quadrature rule is involved:
//   M      = (V V^T)^-1 / 2^dim                  reference mass matrix
//   Dn_u   = (dV/du) V^-1                         nodal derivative matrix
//   D_u    = M^-1 Dn_u^T M                        weak volume operator (M^-1 S_u)
//   LIFT_f = M^-1 E_f Mf                          face lift (Mf = face mass)
// On affine elements these equal the reference's element-by-element quadrature
// of Mesh.cpp:454-466 (mass), 476-489 (stiffness) and 531-536 (surface
// integral) up to rounding.
#pragma once
#include <array>
#include <vector>

namespace dg {

using Bary = std::array<int, 4>;  // integer barycentric coordinates, sum = order

// Nodes of a simplex of the given dimension (1, 2, 3) and order, gmsh order.
std::vector<Bary> simplex_lattice(int dim, int order);

// Nodes of a face (line or triangle) built on three (or two) abstract vertex
// barycentric vectors, in the face's own gmsh order.
std::vector<Bary> face_lattice_on(int fdim, const Bary *verts, int order);

struct RefElement {
    int dim = 0, order = 0;
    int np = 0;      // nodes per element
    int nf = 0;      // faces per element
    int nfp = 0;     // nodes per face
    int nperm = 0;   // face symmetries (2 for lines, 6 for triangles)
    std::vector<Bary> nodes;          // [np]
    std::vector<double> r;            // [np][3] reference coordinates
    std::vector<int> face_verts;      // [nf][3] element-local vertex ids of each face (gmsh order)
    std::vector<int> fmask;           // [nf][nfp] element node at canonical face position
    std::vector<int> perm;            // [nperm][nfp] position in own face list of neighbour position k
    std::vector<int> perm_verts;      // [nperm][3] vertex permutation generating perm
    std::vector<double> mass;         // [np][np]
    std::vector<double> mass_inv;     // [np][np]
    std::vector<double> fmass;        // [nfp][nfp] face mass on the reference face
    std::vector<double> D;            // [dim][np][np]  D_u[i][j]
    std::vector<double> lift;         // [nf][np][nfp]
    std::vector<double> face_r;       // [nfp][2] reference coordinates of face nodes
    // Derivatives of face basis functions 0 and 1 at the first point of the
    // face's Gauss(2*order) rule, used for the reference's normal orientation.
    double face_first_pt[2] = {0, 0};
    double dphi0_first[2] = {0, 0}, dphi1_first[2] = {0, 0};
};

RefElement make_refel(int dim, int order);

// Orthonormal basis helpers, exposed for tests and the face element.
// Evaluates the orthonormal basis (and gradients wrt gmsh reference coords)
// of the simplex of dimension d, order p, at point x (gmsh reference coords).
void ortho_basis(int d, int p, const double *x, double *psi, double *dpsi /*[nb][3] or null*/);
int simplex_np(int d, int p);

// Lagrange basis values and gradients (gmsh reference coordinates) at a point.
void lagrange_eval(int d, int p, const double *x, double *phi, double *dphi /*[np][3] or null*/);

// Small dense LU with partial pivoting; returns false if singular.
bool lu_inverse(std::vector<double> &A, int n);
bool lu_solve(const double *A, double *b, int n);

}  // namespace dg
