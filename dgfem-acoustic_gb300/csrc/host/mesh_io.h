// Raw meshes: what a gmsh .msh file holds and the reference reads through the
// gmsh API (gmsh::open, getElementsByType, getNodesForPhysicalGroup,
// getPhysicalGroups / getPhysicalName; dgalerkin.cpp:24-26, Mesh.cpp:25-38,
// 371, configParser.cpp:117-132).
//
// Readers: MSH 2.2, 4.0 and 4.1 ASCII; MSH 2.2 and 4.1 binary (either byte
// order, data size 4 or 8).  Writer: MSH 4.1 ASCII.
// Generators: structured boxes of straight-sided simplices of any order 1..5,
// with high-order nodes shared between neighbours (as gmsh meshes have them),
// boundary facets grouped per side into physical groups, and optional removed
// cells (obstacles).
#pragma once
#include <string>
#include <vector>

namespace dg {

struct PhysGroup {
    int dim = 0, tag = 0;
    std::string name;
    std::vector<int> nodes;  // sorted unique node tags of the group's elements
};

struct RawMesh {
    int dim = 0;        // model dimension (max entity dimension)
    int el_type = 0;    // gmsh element type of the volume elements
    int order = 0;
    int np = 0;         // nodes per volume element
    std::vector<int> node_tags;   // [nn]
    std::vector<double> xyz;      // [nn][3]
    std::vector<int> el_tags;     // [K]
    std::vector<int> el_nodes;    // [K][np] node tags, gmsh order
    std::vector<PhysGroup> phys;  // all physical groups, ascending (dim, tag)
    // boundary facets, kept for writing: [nb][nbp] node tags and entity id
    int bnd_np = 0;
    std::vector<int> bnd_nodes;
    std::vector<int> bnd_entity;
    std::vector<std::string> entity_names;  // physical name of boundary entity e (1-based ids)
    int num_el() const { return np ? (int)(el_nodes.size() / np) : 0; }
};

// gmsh element type helpers
int gmsh_type(int dim, int order);             // simplex of dim (1,2,3) and order
bool gmsh_type_info(int type, int *dim, int *order, int *np);

// Returns an empty string on success, an error message otherwise.
std::string read_msh(const std::string &path, RawMesh &out);
std::string write_msh(const RawMesh &m, const std::string &path);

// Structured boxes.  side_names: 2D {y=lo, x=hi, y=hi, x=lo}; 3D {x=lo, x=hi,
// y=lo, y=hi, z=lo, z=hi}; obstacle faces use obstacle_name.  removed: cell
// indices (i + nx*(j + ny*k)) that are left out.
std::string box_tri(int nx, int ny, const double lo[2], const double hi[2], int order,
                    const std::vector<std::string> &side_names, RawMesh &out);
std::string box_tet(int nx, int ny, int nz, const double lo[3], const double hi[3], int order,
                    const std::vector<std::string> &side_names, const std::vector<int> &removed,
                    const std::string &obstacle_name, RawMesh &out);

}  // namespace dg
