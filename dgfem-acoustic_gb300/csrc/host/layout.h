// Element-centric device layout built from the reference Mesh arrays
// (dg_mesh_desc): per element the inverse Jacobian, per element face the
// outward normal, detJf/detJe, neighbour, neighbour's local face, face
// permutation, boundary kind and jump sign; plus the reference-element
// operators and tables the stage kernels keep in shared memory.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../../include/dgcuda.h"

namespace dg {

struct Layout {
    int dim = 0, order = 0, np = 0, nf = 0, nfp = 0, nq = 0, nperm = 0, K = 0;
    std::vector<double> geo;     // [K][dim*dim]  B[x][u] = (dx/du)^-1 at x*dim+u
    std::vector<double> fgeo;    // [K][nf][4]    outward normal (dim), detJf/detJe
    std::vector<int> conn;       // [K][nf][2]    neighbour, connectivity word
    std::vector<double> ops;     // D as [u][j][i], then LIFT as [lf*nfp+k][i]
    std::vector<uint8_t> tabs;   // fmask [nf][nfp], perm [nperm][nfp]
    std::vector<double> mass;    // [np][np] reference mass matrix
    std::vector<double> detj;    // [K]
};

// Returns "" or an error message.
std::string build_layout(const dg_mesh_desc &m, int flux_sign, Layout &out);

}  // namespace dg
