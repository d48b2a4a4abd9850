// "Gauss<2p>" integration rules on gmsh's reference simplices (lines on
// [-1, 1], triangles and tetrahedra with a vertex at the origin): the rules
// the reference's Mesh evaluates its per-point geometry on (Mesh.cpp:31-38,
// 135-142).  Tables: rules.inc, written by gen_rules.py.
#pragma once
#include <vector>

namespace dg {

struct QuadRule {
    int n = 0;
    std::vector<double> uvwq;  // [n][4]: u, v, w, weight
};

// dim 1..3, degree 2, 4, 6, 8 or 10; n = 0 if there is no such rule.
QuadRule quad_rule(int dim, int degree);

}  // namespace dg
