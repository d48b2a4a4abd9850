// Element-centric device layout built from the reference Mesh arrays
// (dg_mesh_desc): per element the inverse Jacobian, per element face the
// outward normal, detJf/detJe, neighbour, neighbour's local face, face
// permutation, boundary kind and jump sign; plus the reference-element
// operators and tables the stage kernels keep in shared memory.  Meshes with
// curved elements also get the list of the straight-sided ones, which the
// affine kernels run over, leaving the curved ones to the per-point form.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../../include/dgcuda.h"

namespace dg {

// Curved (non-affine) elements, run by the per-point form: per element the
// inverse mass matrix and the metric terms at the points of the element rule,
// per element face the outward normal and weight x face determinant at the
// points of the face rule, the neighbour and the element nodes of the face's
// nodes on both sides (in the order of the reference's unique face).
struct CurvedLayout {
    int C = 0, ng = 0, ngf = 0;
    std::vector<int> el;          // [C] element ids, ascending
    std::vector<int> slot;        // [K] position in el, or -1
    std::vector<int> affine;      // the other elements, ascending
    std::vector<double> minv;     // [C][np*np] inverse mass, row-major as the reference stores it
    std::vector<double> wm;       // [C][ng][dim*dim] w detJ J^-T at x*dim+u
    std::vector<double> wdet;     // [C][ng] w detJ
    std::vector<double> fw;       // [C][nf][ngf][4] outward normal (dim), w detJf
    std::vector<int> fconn;       // [C][nf][2] neighbour (-1 on the boundary), word (kind, jump sign)
    std::vector<uint8_t> fmap;    // [C][nf][2][nfp] own / neighbour element node of face node k
    std::vector<double> phi;      // [ng][np]
    std::vector<double> dphi;     // [dim][ng][np]
    std::vector<double> fphi;     // [ngf][nfp]
};

struct Layout {
    int dim = 0, order = 0, np = 0, nf = 0, nfp = 0, nq = 0, nperm = 0, K = 0;
    std::vector<double> geo;     // [K][dim*dim]  B[x][u] = (dx/du)^-1 at x*dim+u
    std::vector<double> fgeo;    // [K][nf][4]    outward normal (dim), detJf/detJe
    std::vector<int> conn;       // [K][nf][2]    neighbour, connectivity word
    std::vector<double> ops;     // D as [u][j][i], then LIFT as [lf*nfp+k][i]
    std::vector<uint8_t> tabs;   // fmask [nf][nfp], perm [nperm][nfp]
    std::vector<double> mass;    // [np][np] reference mass matrix
    std::vector<double> detj;    // [K]
    CurvedLayout curved;         // empty for straight-sided meshes
};

// Returns "" or an error message.
std::string build_layout(const dg_mesh_desc &m, int flux_sign, Layout &out);

}  // namespace dg
