// Reference-semantics mesh precompute: the arrays the reference's Mesh
// constructor builds (Mesh.cpp:20-435) that its RK4 right-hand side reads.
// On straight-sided (affine) simplices every per-quadrature-point quantity is
// constant over an element or face and is stored once (at the first point).
// Elements whose nodes are not the affine image of the reference lattice
// (curved, isoparametric elements) are counted; when there is at least one,
// the per-point arrays of the reference (Jacobians and determinants of every
// element at every point of its Gauss(2p) rule, face normals and determinants
// at every face point, basis values and gradients) are filled as well, for
// all elements and faces, in the reference's layouts (Mesh.h:31-108).
//
// Semantics kept from the reference:
//  * unique faces = first occurrence in (element, local face) order, face node
//    order = that first element's local face order (Mesh.cpp:679-713);
//  * face neighbours in ascending element order (Mesh.cpp:235-246);
//  * face-node -> element-node map by node tag (Mesh.cpp:253-263);
//  * face normal from the face basis gradients at the first point of the face
//    Gauss(2p) rule (Mesh.cpp:164-194), with gmsh's completion of the Jacobian
//    of a lower-dimensional element;
//  * orientation = sign((first face node - element barycentre) . n)
//    (Mesh.cpp:278-294); the neighbour swap of Mesh.cpp:302-314 only runs when
//    the mesh has exactly two faces (its condition tests the face count);
//  * boundary normals flipped outward, orientation set to +1 (Mesh.cpp:336-353);
//  * boundary type from the face's first node tag, physical groups processed in
//    ascending tag order (Mesh.cpp:364-384); 1 = reflecting, 0 = absorbing;
//  * fc = -1 for 3D meshes of order > 1 (Mesh.cpp:210-211).
// Face matching uses hashing of sorted face node tags instead of the
// reference's quadratic searches; the result is the same.
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "../../../include/dgcuda.h"
#include "mesh_io.h"
#include "refel.h"

namespace dg {

struct Precomp {
    int dim = 0, order = 0, K = 0, np = 0, F = 0, nf = 0, nfp = 0, fc = 1;
    std::vector<double> el_jac;       // [K][9] dx_x/du_u at [u*3+x], gmsh completion in 2D
    std::vector<double> el_detj;      // [K]
    std::vector<double> f_normal;     // [F][3]
    std::vector<double> f_detj;       // [F]
    std::vector<int> el_f_ids;        // [K][nf]
    std::vector<int> el_f_orient;     // [K][nf]
    std::vector<int> f_nbr;           // [F][2], -1 if none
    std::vector<int> f_n_to_el_n;     // [F][nfp][2], -1 if none
    std::vector<int> f_bc;            // [F]
    std::vector<unsigned char> f_is_bnd;  // [F]
    std::vector<int> f_node_tags;     // [F][nfp]
    std::vector<double> dof_xyz;      // [K*np][3]
    std::vector<int> el_node_tags;    // [K][np]
    // curved elements
    int ncurved = 0;
    std::vector<unsigned char> el_curved;  // [K] node lattice not affine
    int ng = 0, ngf = 0;                // points of the element / face rules
    std::vector<double> el_qp;          // [ng][4] u, v, w, weight
    std::vector<double> el_phi;         // [ng][np]
    std::vector<double> el_dphi;        // [ng][np][3] d/du, d/dv, d/dw
    std::vector<double> el_jac_qp;      // [K][ng][9] dx_x/du_u at [u*3+x]
    std::vector<double> el_detj_qp;     // [K][ng]
    std::vector<double> f_qp;           // [ngf][4]
    std::vector<double> f_phi;          // [ngf][nfp]
    std::vector<double> f_normal_qp;    // [F][ngf][3] after the boundary flip
    std::vector<double> f_detj_qp;      // [F][ngf]
};

// The reference Mesh arrays of a precompute as the solver's descriptor
// (first-point arrays, and the per-point arrays when some element is
// curved); pointers into P, which must outlive the descriptor.
void fill_desc(const Precomp &P, dg_mesh_desc &d);

// physical_bcs: (physical tag, reflecting?) for the boundary groups the
// configuration names, ascending tag order (configParser.cpp:117-132).
std::string precompute(const RawMesh &m, const std::vector<std::pair<int, bool>> &physical_bcs,
                       Precomp &out);

}  // namespace dg
