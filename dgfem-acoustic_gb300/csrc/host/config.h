// .conf parser with the reference's keys and quirks (configParser.cpp:30-150):
// all whitespace removed from each line, '#' comments, key=value (a line
// without '=' maps to itself), std::map key order for sources and initial
// conditions, dipole/quadrupole expansion, numThreads==1 -> 0, the misspelt
// "initialCondtition" prefix, boundary types matched by physical name.
// Keys the reference does not read (precision, fluxSign) select this
// library's options and are ignored by the reference.
#pragma once
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "mesh_io.h"

namespace dg {

struct Config {
    double timeStart = 0, timeEnd = 1, timeStep = 0.1, timeRate = 0.1;
    std::string elementType = "Lagrange";
    std::string timeIntMethod = "Euler1";
    int numThreads = 1;
    double v0[3] = {0, 0, 0};
    double rho0 = 1, c0 = 1;
    // {pole, x, y, z, size, amp, freq, phase, duration}
    std::vector<std::vector<double>> sources;
    // {0, x, y, z, size, amp}
    std::vector<std::vector<double>> initConditions;
    std::string saveFile = "results.msh";
    // physical tag -> reflecting?  (ascending tag order, as std::map)
    std::map<int, bool> physBCs;
    std::vector<std::string> warnings;
    // options of this library
    std::string precision = "fp64";
    std::string fluxSign = "reference";
    std::map<std::string, std::string> raw;
};

// Parses the file; boundary conditions are resolved against the mesh's
// physical groups of dimension mesh.dim-1.  Returns "" or an error message.
std::string parse_config(const std::string &path, const RawMesh &mesh, Config &out);

}  // namespace dg
