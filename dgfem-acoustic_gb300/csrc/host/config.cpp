// .conf parser (see config.h for the reference behaviour kept).
#include "config.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace dg {

namespace {

std::vector<std::string> split(const std::string &s, char d) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string tok;
    while (std::getline(ss, tok, d)) out.push_back(tok);
    return out;
}

// std::stod semantics: leading number prefix, error if nothing converts.
bool to_double(const std::string &s, double &v) {
    if (s.empty()) return false;
    const char *b = s.c_str();
    char *e = nullptr;
    v = std::strtod(b, &e);
    return e != b;
}
bool to_int(const std::string &s, int &v) {
    if (s.empty()) return false;
    const char *b = s.c_str();
    char *e = nullptr;
    long x = std::strtol(b, &e, 10);
    if (e == b) return false;
    v = (int)x;
    return true;
}

}  // namespace

std::string parse_config(const std::string &path, const RawMesh &mesh, Config &c) {
    c = Config();
    std::ifstream f(path);
    if (!f.is_open()) return "cannot open configuration file " + path;
    std::map<std::string, std::string> &cm = c.raw;
    std::string line;
    while (std::getline(f, line)) {
        line.erase(std::remove_if(line.begin(), line.end(), [](unsigned char ch) { return std::isspace(ch); }),
                   line.end());
        if (line.empty() || line[0] == '#') continue;
        size_t pos = line.find('=');
        std::string name = line.substr(0, pos);
        std::string value = line.substr(pos == std::string::npos ? 0 : pos + 1);
        cm[name] = value;
    }
    auto need_d = [&](const char *k, double &v) -> std::string {
        if (!to_double(cm[k], v)) return std::string("configuration key '") + k + "' missing or not a number";
        return "";
    };
    std::string err;
    if (!(err = need_d("timeStart", c.timeStart)).empty()) return err;
    if (!(err = need_d("timeEnd", c.timeEnd)).empty()) return err;
    if (!(err = need_d("timeStep", c.timeStep)).empty()) return err;
    if (!(err = need_d("timeRate", c.timeRate)).empty()) return err;
    // a step that does not advance time would make the time loop
    // (solver.cpp:216, t <= timeEnd; t += timeStep) run forever: refused
    if (!(c.timeStep > 0) || !std::isfinite(c.timeStep))
        return "configuration key 'timeStep' must be a positive number";
    c.elementType = cm["elementType"];
    c.timeIntMethod = cm["timeIntMethod"];
    c.saveFile = cm["saveFile"];
    if (!to_int(cm["numThreads"], c.numThreads)) return "configuration key 'numThreads' missing or not an integer";
    c.numThreads = c.numThreads == 1 ? 0 : c.numThreads;
    if (!(err = need_d("v0_x", c.v0[0])).empty()) return err;
    if (!(err = need_d("v0_y", c.v0[1])).empty()) return err;
    if (!(err = need_d("v0_z", c.v0[2])).empty()) return err;
    if (!(err = need_d("rho0", c.rho0)).empty()) return err;
    if (!(err = need_d("c0", c.c0)).empty()) return err;

    for (auto &kv : cm) {
        const std::string &key = kv.first;
        if (key.find("source") == 0) {
            auto sep = split(kv.second, ',');
            if (sep.size() < 9) return "source '" + key + "' needs 9 comma-separated values";
            double v[8];
            for (int i = 0; i < 8; ++i)
                if (!to_double(sep[i + 1], v[i])) return "source '" + key + "' has a bad number";
            double x = v[0], y = v[1], z = v[2], size = v[3], amp = v[4], freq = v[5], phase = v[6], dur = v[7];
            if (sep[0] == "dipole") {
                c.sources.push_back({1, x - size, y, z, size / 2., amp, freq, phase, dur});
                c.sources.push_back({1, x + size, y, z, size / 2., amp, freq, phase + M_PI, dur});
            } else if (sep[0] == "quadrupole") {
                c.sources.push_back({2, x - size, y, z, size / 2., amp, freq, phase, dur});
                c.sources.push_back({2, x + size, y, z, size / 2., amp, freq, phase, dur});
                c.sources.push_back({2, x, y - size, z, size / 2., amp, freq, phase + M_PI, dur});
                c.sources.push_back({2, x, y + size, z, size / 2., amp, freq, phase + M_PI, dur});
            } else {
                c.sources.push_back({0, x, y, z, size, amp, freq, phase, dur});
            }
        } else if (key.find("initialCondtition") == 0) {
            auto sep = split(kv.second, ',');
            if (sep.size() < 6) return "initial condition '" + key + "' needs 6 comma-separated values";
            double v[5];
            for (int i = 0; i < 5; ++i)
                if (!to_double(sep[i + 1], v[i])) return "initial condition '" + key + "' has a bad number";
            c.initConditions.push_back({0, v[0], v[1], v[2], v[3], v[4]});
        }
    }
    for (auto &pg : mesh.phys) {
        if (pg.dim != mesh.dim - 1) continue;
        const std::string &val = cm[pg.name];
        if (val.find("Absorbing") == 0) c.physBCs[pg.tag] = false;
        else if (val.find("Reflecting") == 0) c.physBCs[pg.tag] = true;
        else c.warnings.push_back("Not specified or supported boundary conditions.");
    }
    if (cm.count("precision")) c.precision = cm["precision"];
    if (cm.count("fluxSign")) c.fluxSign = cm["fluxSign"];
    return "";
}

}  // namespace dg
