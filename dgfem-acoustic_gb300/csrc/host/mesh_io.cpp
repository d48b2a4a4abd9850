// Raw mesh reading, writing and generation.
#include "mesh_io.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

#include "refel.h"

namespace dg {

int gmsh_type(int dim, int order) {
    static const int line[6] = {0, 1, 8, 26, 27, 28};
    static const int tri[6] = {0, 2, 9, 21, 23, 25};
    static const int tet[6] = {0, 4, 11, 29, 30, 31};
    if (order < 1 || order > 5) return -1;
    if (dim == 1) return line[order];
    if (dim == 2) return tri[order];
    if (dim == 3) return tet[order];
    return -1;
}

bool gmsh_type_info(int type, int *dim, int *order, int *np) {
    for (int d = 1; d <= 3; ++d)
        for (int p = 1; p <= 5; ++p)
            if (gmsh_type(d, p) == type) {
                *dim = d;
                *order = p;
                *np = simplex_np(d, p);
                return true;
            }
    if (type == 15) { *dim = 0; *order = 0; *np = 1; return true; }
    return false;
}

namespace {

// Whole-file tokenizer
struct Tok {
    std::string buf;
    size_t pos = 0;
    bool load(const std::string &path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) return false;
        std::ostringstream ss;
        ss << f.rdbuf();
        buf = ss.str();
        return true;
    }
    void skip_ws() {
        while (pos < buf.size() && (unsigned char)buf[pos] <= ' ') ++pos;
    }
    bool eof() { skip_ws(); return pos >= buf.size(); }
    std::string word() {
        skip_ws();
        size_t s = pos;
        while (pos < buf.size() && (unsigned char)buf[pos] > ' ') ++pos;
        return buf.substr(s, pos - s);
    }
    long integer() {
        skip_ws();
        char *end;
        long v = std::strtol(buf.c_str() + pos, &end, 10);
        if (end == buf.c_str() + pos) throw std::runtime_error("expected integer");
        pos = end - buf.c_str();
        return v;
    }
    double real() {
        skip_ws();
        char *end;
        double v = std::strtod(buf.c_str() + pos, &end);
        if (end == buf.c_str() + pos) throw std::runtime_error("expected number");
        pos = end - buf.c_str();
        return v;
    }
    std::string quoted() {
        skip_ws();
        if (pos < buf.size() && buf[pos] == '"') {
            size_t e = buf.find('"', pos + 1);
            if (e == std::string::npos) throw std::runtime_error("unterminated quoted string");
            std::string s = buf.substr(pos + 1, e - pos - 1);
            pos = e + 1;
            return s;
        }
        return word();
    }
    void skip_to(const std::string &end_marker) {
        size_t e = buf.find(end_marker, pos);
        pos = (e == std::string::npos) ? buf.size() : e + end_marker.size();
    }

    // Binary files (MSH 4.1 and 2.2, file-type 1): section names, counts of
    // MSH 2.2 and $PhysicalNames stay ASCII; the section data that follows
    // the line end is raw: int = 4 bytes, size_t = data-size bytes, double =
    // 8 bytes, in the byte order of the file's endianness marker.
    bool bin = false, swap = false;
    int dsize = 8;
    void line_end() {  // the end of the ASCII line before raw data
        while (pos < buf.size() && (buf[pos] == ' ' || buf[pos] == '\t' || buf[pos] == '\r')) ++pos;
        if (pos < buf.size() && buf[pos] == '\n') ++pos;
    }
    template <typename T>
    T raw() {
        if (pos + sizeof(T) > buf.size()) throw std::runtime_error("truncated binary data");
        T v;
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    uint32_t raw32() {
        uint32_t v = raw<uint32_t>();
        return swap ? __builtin_bswap32(v) : v;
    }
    uint64_t raw64() {
        uint64_t v = raw<uint64_t>();
        return swap ? __builtin_bswap64(v) : v;
    }
    // a count read from the file: each item takes at least min_bytes of what
    // is left, so larger counts are corrupt (and must not size an allocation)
    long count(long n, long min_bytes) {
        const long left = (long)(buf.size() - std::min(pos, buf.size()));
        if (n < 0 || n > left / std::max(1L, min_bytes)) throw std::runtime_error("count exceeds the file");
        return n;
    }
    // fields by their type in the format: ASCII tokens or raw values
    long I() { return bin ? (long)(int32_t)raw32() : integer(); }
    long S() {
        if (!bin) return integer();
        const uint64_t v = dsize == 8 ? raw64() : (uint64_t)raw32();
        if (v > (uint64_t)INT32_MAX) throw std::runtime_error("count or tag too large");
        return (long)v;
    }
    double R() {
        if (!bin) return real();
        const uint64_t v = raw64();
        double d;
        std::memcpy(&d, &v, 8);
        return d;
    }
};

struct ElemBlock {
    int ent_dim, ent_tag, type;
    std::vector<int> tags;
    std::vector<int> nodes;
};

}  // namespace

std::string read_msh(const std::string &path, RawMesh &out) {
    Tok t;
    if (!t.load(path)) return "cannot open mesh file " + path;
    out = RawMesh();
    double version = 0;
    std::map<int, std::string> names_by_tag[4];
    // entity (dim, tag) -> physical tags
    std::map<std::pair<int, int>, std::vector<int>> ent_phys;
    std::vector<ElemBlock> blocks;
    std::vector<std::pair<int, std::array<double, 3>>> nodes;
    int max_ent_dim = -1;
    try {
        while (!t.eof()) {
            std::string sec = t.word();
            if (sec == "$MeshFormat") {
                version = t.real();
                int ft = (int)t.integer();
                int ds = (int)t.integer();
                if (ft == 1) {
                    if (version >= 4.0 && version < 4.1) return "binary MSH 4.0 files are not supported";
                    if (ds != 4 && ds != 8) return "unsupported data size " + std::to_string(ds);
                    t.bin = true;
                    t.dsize = ds;
                    t.line_end();
                    const uint32_t one = t.raw<uint32_t>();
                    if (one == 1u) t.swap = false;
                    else if (__builtin_bswap32(one) == 1u) t.swap = true;
                    else return "bad endianness marker in " + path;
                } else if (ft != 0) {
                    return "unknown file type " + std::to_string(ft);
                }
                t.skip_to("$EndMeshFormat");
            } else if (sec == "$PhysicalNames") {
                long n = t.count(t.integer(), 6);
                for (long i = 0; i < n; ++i) {
                    int d = (int)t.integer();
                    int tag = (int)t.integer();
                    if (d < 0 || d > 3) return "invalid physical group dimension " + std::to_string(d) + " in " + path;
                    names_by_tag[d][tag] = t.quoted();
                }
                t.skip_to("$EndPhysicalNames");
            } else if (sec == "$Entities" && version >= 4.0) {
                if (t.bin) t.line_end();
                long cnt[4];
                for (int d = 0; d < 4; ++d) cnt[d] = t.count(t.S(), 4);
                for (int d = 0; d < 4; ++d)
                    for (long e = 0; e < cnt[d]; ++e) {
                        int tag = (int)t.I();
                        int ncoord = (d == 0 && version >= 4.1) ? 3 : 6;
                        for (int k = 0; k < ncoord; ++k) t.R();
                        long nph = t.count(t.S(), 1);
                        std::vector<int> ph;
                        for (long k = 0; k < nph; ++k) ph.push_back((int)t.I());
                        ent_phys[{d, tag}] = ph;
                        if (d > 0) {
                            long nb = t.count(t.S(), 1);
                            for (long k = 0; k < nb; ++k) t.I();
                        }
                        if (cnt[d] > 0) max_ent_dim = std::max(max_ent_dim, d);
                    }
                t.skip_to("$EndEntities");
            } else if (sec == "$Nodes") {
                if (version >= 4.0) {
                    if (t.bin) t.line_end();
                    long nblk = t.count(t.S(), 4);
                    long nn = t.count(t.S(), 4);
                    if (version >= 4.1) { t.S(); t.S(); }
                    nodes.reserve(nn);
                    for (long b = 0; b < nblk; ++b) {
                        long a0 = t.I(), a1 = t.I();
                        const int edim = (int)(version >= 4.1 ? a0 : a1);
                        int param = (int)t.I();
                        long n = t.count(t.S(), 4);
                        // parametric blocks add the node's entityDim
                        // parametric coordinates after x y z (skipped)
                        const int npar = param ? std::max(0, std::min(edim, 3)) : 0;
                        if (version >= 4.1) {
                            std::vector<int> tags(n);
                            for (long i = 0; i < n; ++i) tags[i] = (int)t.S();
                            for (long i = 0; i < n; ++i) {
                                const double x0 = t.R(), x1 = t.R(), x2 = t.R();
                                for (int k = 0; k < npar; ++k) t.R();
                                nodes.push_back({tags[i], {x0, x1, x2}});
                            }
                        } else {
                            for (long i = 0; i < n; ++i) {
                                int tag = (int)t.integer();
                                std::array<double, 3> x{t.real(), t.real(), t.real()};
                                for (int k = 0; k < npar; ++k) t.real();
                                nodes.push_back({tag, x});
                            }
                        }
                    }
                } else {
                    long nn = t.count(t.integer(), 4);  // ASCII in binary files too
                    if (t.bin) t.line_end();
                    nodes.reserve(nn);
                    for (long i = 0; i < nn; ++i) {
                        int tag = (int)t.I();
                        const double x0 = t.R(), x1 = t.R(), x2 = t.R();
                        nodes.push_back({tag, {x0, x1, x2}});
                    }
                }
                t.skip_to("$EndNodes");
            } else if (sec == "$Elements") {
                if (version >= 4.0) {
                    if (t.bin) t.line_end();
                    long nblk = t.count(t.S(), 4);
                    t.S();
                    if (version >= 4.1) { t.S(); t.S(); }
                    for (long b = 0; b < nblk; ++b) {
                        ElemBlock eb;
                        long a0 = t.I(), a1 = t.I();
                        if (version >= 4.1) { eb.ent_dim = (int)a0; eb.ent_tag = (int)a1; }
                        else { eb.ent_tag = (int)a0; eb.ent_dim = (int)a1; }
                        eb.type = (int)t.I();
                        long n = t.S();
                        int d, p, np;
                        if (!gmsh_type_info(eb.type, &d, &p, &np))
                            return "unsupported element type " + std::to_string(eb.type);
                        if (eb.ent_dim != d)
                            return "element block of dimension " + std::to_string(eb.ent_dim) + " holds type " +
                                   std::to_string(eb.type) + " in " + path;
                        t.count(n, 2L * (np + 1));
                        eb.tags.resize(n);
                        eb.nodes.resize(n * np);
                        for (long i = 0; i < n; ++i) {
                            eb.tags[i] = (int)t.S();
                            for (int k = 0; k < np; ++k) eb.nodes[i * np + k] = (int)t.S();
                        }
                        blocks.push_back(std::move(eb));
                    }
                } else {
                    long ne = t.count(t.integer(), 4);  // ASCII in binary files too
                    if (t.bin) t.line_end();
                    // MSH2: group per (type, physical, elementary); binary
                    // files give the elements in runs of one type and tag
                    // count (header: type, run length, tag count)
                    std::map<std::array<int, 3>, size_t> idx;
                    long run = 0;
                    int run_type = 0, run_ntags = 0;
                    for (long i = 0; i < ne; ++i) {
                        int tag, type, ntags;
                        if (t.bin) {
                            if (run == 0) {
                                run_type = (int)t.I();
                                run = t.I();
                                run_ntags = (int)t.I();
                                if (run < 1 || run_ntags < 0) return "bad element run header in " + path;
                            }
                            --run;
                            tag = (int)t.I();
                            type = run_type;
                            ntags = run_ntags;
                        } else {
                            tag = (int)t.integer();
                            type = (int)t.integer();
                            ntags = (int)t.integer();
                        }
                        int phys = 0, elem = 0;
                        for (int k = 0; k < ntags; ++k) {
                            int v = (int)t.I();
                            if (k == 0) phys = v;
                            if (k == 1) elem = v;
                        }
                        int d, p, np;
                        if (!gmsh_type_info(type, &d, &p, &np))
                            return "unsupported element type " + std::to_string(type);
                        // MSH2 has no entities: synthesise one entity per (dim, elementary)
                        std::array<int, 3> key{type, elem, phys};
                        auto it = idx.find(key);
                        if (it == idx.end()) {
                            ElemBlock eb;
                            eb.ent_dim = d;
                            eb.ent_tag = elem;
                            eb.type = type;
                            idx[key] = blocks.size();
                            blocks.push_back(eb);
                            it = idx.find(key);
                            auto &ph = ent_phys[{d, elem}];
                            if (phys && std::find(ph.begin(), ph.end(), phys) == ph.end()) ph.push_back(phys);
                        }
                        ElemBlock &eb = blocks[it->second];
                        eb.tags.push_back(tag);
                        for (int k = 0; k < np; ++k) eb.nodes.push_back((int)t.I());
                        max_ent_dim = std::max(max_ent_dim, d);
                    }
                }
                t.skip_to("$EndElements");
            } else if (!sec.empty() && sec[0] == '$') {
                std::string end = "$End" + sec.substr(1);
                t.skip_to(end);
            } else {
                // quote at most 32 bytes of the token, non-printable ones as '?'
                std::string shown;
                for (size_t k = 0; k < sec.size() && k < 32; ++k)
                    shown += (sec[k] >= 0x20 && sec[k] < 0x7f) ? sec[k] : '?';
                return "unexpected token '" + shown + (sec.size() > 32 ? "...'" : "'") + " in " + path;
            }
        }
    } catch (std::exception &e) {
        return std::string("parse error in ") + path + ": " + e.what();
    }
    if (blocks.empty()) return "no elements in " + path;
    for (auto &b : blocks) max_ent_dim = std::max(max_ent_dim, b.ent_dim);
    out.dim = max_ent_dim;
    if (out.dim < 2) return "only 2D and 3D meshes are supported";
    // nodes
    std::sort(nodes.begin(), nodes.end(),
              [](const std::pair<int, std::array<double, 3>> &a, const std::pair<int, std::array<double, 3>> &b) {
                  return a.first < b.first;
              });
    // gmsh tags start at 1; a node tag may appear once
    for (size_t i = 0; i < nodes.size(); ++i) {
        if (nodes[i].first < 1) return "invalid node tag " + std::to_string(nodes[i].first) + " in " + path;
        if (i > 0 && nodes[i].first == nodes[i - 1].first)
            return "duplicate node tag " + std::to_string(nodes[i].first) + " in " + path;
    }
    for (auto &b : blocks)
        for (int t : b.nodes)
            if (t < 1) return "invalid element node tag " + std::to_string(t) + " in " + path;
    out.node_tags.resize(nodes.size());
    out.xyz.resize(nodes.size() * 3);
    for (size_t i = 0; i < nodes.size(); ++i) {
        out.node_tags[i] = nodes[i].first;
        for (int k = 0; k < 3; ++k) out.xyz[i * 3 + k] = nodes[i].second[k];
    }
    // volume elements: blocks of the top dimension, ordered by entity tag
    std::stable_sort(blocks.begin(), blocks.end(), [](const ElemBlock &a, const ElemBlock &b) {
        if (a.ent_dim != b.ent_dim) return a.ent_dim < b.ent_dim;
        return a.ent_tag < b.ent_tag;
    });
    for (auto &b : blocks) {
        int d, p, np;
        gmsh_type_info(b.type, &d, &p, &np);
        if (b.ent_dim != out.dim || d != out.dim) continue;
        if (out.el_type == 0) { out.el_type = b.type; out.order = p; out.np = np; }
        if (b.type != out.el_type) return "meshes with more than one element type are not supported";
        out.el_tags.insert(out.el_tags.end(), b.tags.begin(), b.tags.end());
        out.el_nodes.insert(out.el_nodes.end(), b.nodes.begin(), b.nodes.end());
    }
    if (out.el_type == 0) return "no volume elements";
    // physical groups and their nodes
    std::map<std::pair<int, int>, std::set<int>> grp_nodes;
    for (auto &b : blocks) {
        auto it = ent_phys.find({b.ent_dim, b.ent_tag});
        if (it == ent_phys.end()) continue;
        for (int ph : it->second) {
            auto &s = grp_nodes[{b.ent_dim, ph}];
            s.insert(b.nodes.begin(), b.nodes.end());
        }
    }
    std::set<std::pair<int, int>> all_groups;
    for (auto &kv : grp_nodes) all_groups.insert(kv.first);
    for (int d = 0; d < 4; ++d)
        for (auto &kv : names_by_tag[d]) all_groups.insert({d, kv.first});
    for (auto &g : all_groups) {
        PhysGroup pg;
        pg.dim = g.first;
        pg.tag = g.second;
        auto nit = names_by_tag[g.first].find(g.second);
        if (nit != names_by_tag[g.first].end()) pg.name = nit->second;
        auto sit = grp_nodes.find(g);
        if (sit != grp_nodes.end()) pg.nodes.assign(sit->second.begin(), sit->second.end());
        out.phys.push_back(pg);
    }
    // boundary facets (for rewriting)
    int bt = gmsh_type(out.dim - 1, out.order);
    int d, p, bnp;
    gmsh_type_info(bt, &d, &p, &bnp);
    out.bnd_np = bnp;
    std::map<int, int> ent_id;
    for (auto &b : blocks) {
        if (b.ent_dim != out.dim - 1 || b.type != bt) continue;
        int eid;
        auto it = ent_id.find(b.ent_tag);
        if (it == ent_id.end()) {
            eid = (int)ent_id.size() + 1;
            ent_id[b.ent_tag] = eid;
            std::string nm;
            auto pit = ent_phys.find({b.ent_dim, b.ent_tag});
            if (pit != ent_phys.end() && !pit->second.empty()) {
                auto nit = names_by_tag[b.ent_dim].find(pit->second[0]);
                if (nit != names_by_tag[b.ent_dim].end()) nm = nit->second;
            }
            out.entity_names.push_back(nm);
        } else {
            eid = it->second;
        }
        out.bnd_nodes.insert(out.bnd_nodes.end(), b.nodes.begin(), b.nodes.end());
        for (size_t i = 0; i < b.tags.size(); ++i) out.bnd_entity.push_back(eid);
    }
    return "";
}

std::string write_msh(const RawMesh &m, const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return "cannot write " + path;
    int nb_ent = (int)m.entity_names.size();
    // physical names: unique boundary names, then the domain
    std::vector<std::string> bnames;
    for (auto &n : m.entity_names)
        if (!n.empty() && std::find(bnames.begin(), bnames.end(), n) == bnames.end()) bnames.push_back(n);
    std::fprintf(f, "$MeshFormat\n4.1 0 8\n$EndMeshFormat\n");
    std::fprintf(f, "$PhysicalNames\n%d\n", (int)bnames.size() + 1);
    for (size_t i = 0; i < bnames.size(); ++i)
        std::fprintf(f, "%d %d \"%s\"\n", m.dim - 1, (int)i + 1, bnames[i].c_str());
    std::fprintf(f, "%d %d \"Domain\"\n", m.dim, (int)bnames.size() + 1);
    std::fprintf(f, "$EndPhysicalNames\n");
    std::fprintf(f, "$Entities\n");
    if (m.dim == 2) std::fprintf(f, "0 %d 1 0\n", nb_ent);
    else std::fprintf(f, "0 0 %d 1\n", nb_ent);
    for (int e = 0; e < nb_ent; ++e) {
        int ph = 0;
        for (size_t i = 0; i < bnames.size(); ++i)
            if (bnames[i] == m.entity_names[e]) ph = (int)i + 1;
        if (ph) std::fprintf(f, "%d 0 0 0 0 0 0 1 %d 0\n", e + 1, ph);
        else std::fprintf(f, "%d 0 0 0 0 0 0 0 0\n", e + 1);
    }
    std::fprintf(f, "1 0 0 0 0 0 0 1 %d 0\n", (int)bnames.size() + 1);
    std::fprintf(f, "$EndEntities\n");
    size_t nn = m.node_tags.size();
    int mint = nn ? *std::min_element(m.node_tags.begin(), m.node_tags.end()) : 0;
    int maxt = nn ? *std::max_element(m.node_tags.begin(), m.node_tags.end()) : 0;
    std::fprintf(f, "$Nodes\n1 %zu %d %d\n%d 1 0 %zu\n", nn, mint, maxt, m.dim, nn);
    for (size_t i = 0; i < nn; ++i) std::fprintf(f, "%d\n", m.node_tags[i]);
    for (size_t i = 0; i < nn; ++i)
        std::fprintf(f, "%.17g %.17g %.17g\n", m.xyz[i * 3], m.xyz[i * 3 + 1], m.xyz[i * 3 + 2]);
    std::fprintf(f, "$EndNodes\n");
    size_t nbnd = m.bnd_np ? m.bnd_nodes.size() / m.bnd_np : 0;
    size_t K = m.num_el();
    // one block per boundary entity + the volume block
    std::vector<std::vector<size_t>> per_ent(nb_ent);
    for (size_t i = 0; i < nbnd; ++i) per_ent[m.bnd_entity[i] - 1].push_back(i);
    int nblocks = 0;
    for (auto &v : per_ent) nblocks += v.empty() ? 0 : 1;
    nblocks += 1;
    size_t ntot = nbnd + K;
    std::fprintf(f, "$Elements\n%d %zu 1 %zu\n", nblocks, ntot, ntot);
    size_t etag = 1;
    int btype = gmsh_type(m.dim - 1, m.order);
    for (int e = 0; e < nb_ent; ++e) {
        if (per_ent[e].empty()) continue;
        std::fprintf(f, "%d %d %d %zu\n", m.dim - 1, e + 1, btype, per_ent[e].size());
        for (size_t i : per_ent[e]) {
            std::fprintf(f, "%zu", etag++);
            for (int k = 0; k < m.bnd_np; ++k) std::fprintf(f, " %d", m.bnd_nodes[i * m.bnd_np + k]);
            std::fprintf(f, "\n");
        }
    }
    std::fprintf(f, "%d 1 %d %zu\n", m.dim, m.el_type, K);
    for (size_t i = 0; i < K; ++i) {
        std::fprintf(f, "%d", m.el_tags.empty() ? (int)etag : m.el_tags[i]);
        ++etag;
        for (int k = 0; k < m.np; ++k) std::fprintf(f, " %d", m.el_nodes[i * m.np + k]);
        std::fprintf(f, "\n");
    }
    std::fprintf(f, "$EndElements\n");
    std::fclose(f);
    return "";
}

namespace {

// Shared part of the generators: elements given as lists of integer lattice
// vertices; lattice node positions X = sum_m n_m V_m (units of h/order).
struct LatticeBuilder {
    int dim, order, np;
    std::vector<Bary> tmpl;  // element node template (barycentric)
    long NX, NY, NZ;         // lattice extents (points per axis)
    std::vector<int> lat_tag;  // lattice index -> node tag (0 = unused)
    std::vector<long> el_lat;  // [K][np] lattice indices
    LatticeBuilder(int d, int p, long nx, long ny, long nz) : dim(d), order(p) {
        tmpl = simplex_lattice(d, p);
        np = (int)tmpl.size();
        NX = nx * p + 1;
        NY = ny * p + 1;
        NZ = (d == 3) ? nz * p + 1 : 1;
    }
    void add(const std::array<std::array<long, 3>, 4> &V) {
        for (int i = 0; i < np; ++i) {
            long X[3] = {0, 0, 0};
            for (int m = 0; m <= dim; ++m)
                for (int k = 0; k < 3; ++k) X[k] += tmpl[i][m] * V[m][k];
            el_lat.push_back(X[0] + NX * (X[1] + NY * X[2]));
        }
    }
};

long orient3(const std::array<std::array<long, 3>, 4> &V) {
    long a[3], b[3], c[3];
    for (int k = 0; k < 3; ++k) { a[k] = V[1][k] - V[0][k]; b[k] = V[2][k] - V[0][k]; c[k] = V[3][k] - V[0][k]; }
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
}

std::string finish(LatticeBuilder &lb, const double *lo, const double *hi, long nx, long ny, long nz,
                   const std::vector<std::string> &side_names, const std::string &obstacle_name, RawMesh &out) {
    out = RawMesh();
    out.dim = lb.dim;
    out.order = lb.order;
    out.np = lb.np;
    out.el_type = gmsh_type(lb.dim, lb.order);
    long nlat = lb.NX * lb.NY * lb.NZ;
    std::vector<int> tag(nlat, 0);
    for (long l : lb.el_lat) tag[l] = 1;
    int next = 1;
    for (long l = 0; l < nlat; ++l)
        if (tag[l]) tag[l] = next++;
    out.node_tags.resize(next - 1);
    out.xyz.resize((next - 1) * 3);
    long ncell[3] = {nx * lb.order, ny * lb.order, (lb.dim == 3 ? nz : 1) * lb.order};
    for (long l = 0; l < nlat; ++l) {
        if (!tag[l]) continue;
        long X = l % lb.NX, Y = (l / lb.NX) % lb.NY, Z = l / (lb.NX * lb.NY);
        int t = tag[l];
        out.node_tags[t - 1] = t;
        long L[3] = {X, Y, Z};
        for (int k = 0; k < 3; ++k) {
            if (k < lb.dim) out.xyz[(t - 1) * 3 + k] = lo[k] + (hi[k] - lo[k]) * double(L[k]) / double(ncell[k]);
            else out.xyz[(t - 1) * 3 + k] = 0.0;
        }
    }
    long K = (long)lb.el_lat.size() / lb.np;
    out.el_nodes.resize(lb.el_lat.size());
    for (size_t i = 0; i < lb.el_lat.size(); ++i) out.el_nodes[i] = tag[lb.el_lat[i]];
    out.el_tags.resize(K);
    // Boundary facets: element faces seen once.
    RefElement re = make_refel(lb.dim, lb.order);
    int nf = re.nf, nfp = re.nfp, nv = lb.dim;
    struct FK { std::array<int, 3> key; long el; int lf; };
    std::vector<FK> fk;
    fk.reserve(K * nf);
    for (long e = 0; e < K; ++e)
        for (int f = 0; f < nf; ++f) {
            std::array<int, 3> key{0, 0, 0};
            for (int k = 0; k < nv; ++k) key[k] = out.el_nodes[e * lb.np + re.face_verts[f * 3 + k]];
            std::sort(key.begin(), key.begin() + nv);
            fk.push_back({key, e, f});
        }
    std::sort(fk.begin(), fk.end(), [](const FK &a, const FK &b) {
        if (a.key != b.key) return a.key < b.key;
        if (a.el != b.el) return a.el < b.el;
        return a.lf < b.lf;
    });
    // entity ids: one per side, then obstacles
    int nsides = (lb.dim == 2) ? 4 : 6;
    std::vector<int> side_ent(nsides + 1, 0);
    std::vector<std::vector<int>> bnodes(nsides + 1);
    out.bnd_np = nfp;
    for (size_t i = 0; i < fk.size();) {
        size_t j = i + 1;
        while (j < fk.size() && fk[j].key == fk[i].key) ++j;
        if (j - i == 1) {
            long e = fk[i].el;
            int f = fk[i].lf;
            // which side: all face vertices share a boundary plane coordinate
            int side = nsides;  // obstacle by default
            long lat[3][3];
            for (int k = 0; k < nv; ++k) {
                long l = lb.el_lat[e * lb.np + re.face_verts[f * 3 + k]];
                lat[k][0] = l % lb.NX;
                lat[k][1] = (l / lb.NX) % lb.NY;
                lat[k][2] = l / (lb.NX * lb.NY);
            }
            auto all_eq = [&](int ax, long v) {
                for (int k = 0; k < nv; ++k)
                    if (lat[k][ax] != v) return false;
                return true;
            };
            if (lb.dim == 2) {
                if (all_eq(1, 0)) side = 0;
                else if (all_eq(0, lb.NX - 1)) side = 1;
                else if (all_eq(1, lb.NY - 1)) side = 2;
                else if (all_eq(0, 0)) side = 3;
            } else {
                if (all_eq(0, 0)) side = 0;
                else if (all_eq(0, lb.NX - 1)) side = 1;
                else if (all_eq(1, 0)) side = 2;
                else if (all_eq(1, lb.NY - 1)) side = 3;
                else if (all_eq(2, 0)) side = 4;
                else if (all_eq(2, lb.NZ - 1)) side = 5;
            }
            for (int k = 0; k < nfp; ++k)
                bnodes[side].push_back(out.el_nodes[e * lb.np + re.fmask[f * nfp + k]]);
        }
        i = j;
    }
    for (int s = 0; s <= nsides; ++s) {
        if (bnodes[s].empty()) continue;
        std::string nm = (s < nsides) ? (s < (int)side_names.size() ? side_names[s] : "") : obstacle_name;
        out.entity_names.push_back(nm);
        int eid = (int)out.entity_names.size();
        out.bnd_nodes.insert(out.bnd_nodes.end(), bnodes[s].begin(), bnodes[s].end());
        for (size_t i = 0; i < bnodes[s].size() / nfp; ++i) out.bnd_entity.push_back(eid);
    }
    // element tags after the boundary facets, like a gmsh file written above
    int etag = (int)out.bnd_entity.size() + 1;
    for (long e = 0; e < K; ++e) out.el_tags[e] = etag++;
    // physical groups: unique boundary names (dim-1), then the domain
    std::vector<std::string> bnames;
    for (auto &n : out.entity_names)
        if (!n.empty() && std::find(bnames.begin(), bnames.end(), n) == bnames.end()) bnames.push_back(n);
    for (size_t i = 0; i < bnames.size(); ++i) {
        PhysGroup pg;
        pg.dim = lb.dim - 1;
        pg.tag = (int)i + 1;
        pg.name = bnames[i];
        std::set<int> s;
        for (size_t b = 0; b < out.bnd_entity.size(); ++b)
            if (out.entity_names[out.bnd_entity[b] - 1] == bnames[i])
                s.insert(out.bnd_nodes.begin() + b * nfp, out.bnd_nodes.begin() + (b + 1) * nfp);
        pg.nodes.assign(s.begin(), s.end());
        out.phys.push_back(pg);
    }
    PhysGroup dom;
    dom.dim = lb.dim;
    dom.tag = (int)bnames.size() + 1;
    dom.name = "Domain";
    {
        std::vector<int> v(out.el_nodes.begin(), out.el_nodes.end());
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        dom.nodes = v;
    }
    out.phys.push_back(dom);
    std::sort(out.phys.begin(), out.phys.end(), [](const PhysGroup &a, const PhysGroup &b) {
        if (a.dim != b.dim) return a.dim < b.dim;
        return a.tag < b.tag;
    });
    return "";
}

}  // namespace

std::string box_tri(int nx, int ny, const double lo[2], const double hi[2], int order,
                    const std::vector<std::string> &side_names, RawMesh &out) {
    if (nx < 1 || ny < 1 || order < 1 || order > 5) return "bad box parameters";
    // element nodes are indexed with 32-bit integers
    if ((long long)nx * ny * 2 * ((order + 1) * (order + 2) / 2) > INT32_MAX) return "box too large";
    LatticeBuilder lb(2, order, nx, ny, 1);
    lb.el_lat.reserve((size_t)nx * ny * 2 * lb.np);
    for (long j = 0; j < ny; ++j)
        for (long i = 0; i < nx; ++i) {
            std::array<long, 3> c00{i, j, 0}, c10{i + 1, j, 0}, c11{i + 1, j + 1, 0}, c01{i, j + 1, 0};
            lb.add({c00, c10, c11, {0, 0, 0}});
            lb.add({c00, c11, c01, {0, 0, 0}});
        }
    double lo3[3] = {lo[0], lo[1], 0}, hi3[3] = {hi[0], hi[1], 0};
    return finish(lb, lo3, hi3, nx, ny, 1, side_names, "", out);
}

std::string box_tet(int nx, int ny, int nz, const double lo[3], const double hi[3], int order,
                    const std::vector<std::string> &side_names, const std::vector<int> &removed,
                    const std::string &obstacle_name, RawMesh &out) {
    if (nx < 1 || ny < 1 || nz < 1 || order < 1 || order > 5) return "bad box parameters";
    // element nodes are indexed with 32-bit integers
    if ((long long)nx * ny * nz * 6 * ((order + 1) * (order + 2) * (order + 3) / 6) > INT32_MAX) return "box too large";
    std::vector<char> gone((size_t)nx * ny * nz, 0);
    for (int c : removed)
        if (c >= 0 && (size_t)c < gone.size()) gone[c] = 1;
    LatticeBuilder lb(3, order, nx, ny, nz);
    static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    lb.el_lat.reserve((size_t)nx * ny * nz * 6 * lb.np);
    for (long k = 0; k < nz; ++k)
        for (long j = 0; j < ny; ++j)
            for (long i = 0; i < nx; ++i) {
                if (gone[i + (size_t)nx * (j + (size_t)ny * k)]) continue;
                for (auto &pm : perms) {
                    std::array<std::array<long, 3>, 4> V;
                    std::array<long, 3> x{i, j, k};
                    V[0] = x;
                    for (int s = 0; s < 3; ++s) {
                        x[pm[s]] += 1;
                        V[s + 1] = x;
                    }
                    if (orient3(V) < 0) std::swap(V[1], V[2]);
                    lb.add(V);
                }
            }
    return finish(lb, lo, hi, nx, ny, nz, side_names, obstacle_name, out);
}

}  // namespace dg
