// dgalerkin mesh.msh config.conf -- the reference's command line
// (src/dgalerkin.cpp:11-63) on the GB300 path.
//
// Same flow: read the mesh and the configuration, build the Mesh
// precompute, set the Gaussian initial conditions (dgalerkin.cpp:37-50), run
// the time loop of solver::rungeKutta (src/solver.cpp:216-286) with its
// t / tDisplay accumulation and save cadence, and write the Pressure,
// Density (p / c0^2) and Velocity views as ElementNodeData to saveFile
// (solver.cpp:185-191, 225-238, 289-291).  The right-hand side runs through
// the C ABI of include/dgcuda.h; steps between two saves are one
// dg_rk4_steps call.  Options the reference does not read: precision
// (fp64 | fp32 | mixed | tf32x3) and fluxSign (reference | upwind) in the .conf.
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../../include/dgcuda.h"
#include "config.h"
#include "mesh_io.h"
#include "precompute.h"

namespace {

// A saved frame: the state [4][ndof] in pinned host memory (dg_host_alloc),
// filled by dg_get_state_async while the next steps run; `ticket` is waited
// for before the views are written.  `own` is the pageable fallback when no
// pinned memory can be had.
struct Frame {
    double t;
    int step;
    double *u = nullptr;
    long long ticket = -1;
    std::vector<double> own;
};

void log(const std::string &s) { std::printf("Info    : %s\n", s.c_str()); }

bool write_views(const std::string &path, const dg::RawMesh &mesh, const dg::Precomp &pre, const dg::Config &cfg,
                 const std::vector<Frame> &frames) {
    std::string err = dg::write_msh(mesh, path);
    if (!err.empty()) {
        std::fprintf(stderr, "Error   : %s\n", err.c_str());
        return false;
    }
    FILE *f = std::fopen(path.c_str(), "a");
    if (!f) return false;
    const int K = pre.K, np = pre.np;
    const size_t ndof = (size_t)K * np;
    const char *names[3] = {"Pressure", "Density", "Velocity"};
    for (int v = 0; v < 3; ++v) {
        for (const Frame &fr : frames) {
            int ncomp = v == 2 ? 3 : 1;
            std::fprintf(f, "$ElementNodeData\n1\n\"%s\"\n1\n%.17g\n3\n%d\n%d\n%d\n", names[v], fr.t, fr.step, ncomp,
                         K);
            for (int e = 0; e < K; ++e) {
                std::fprintf(f, "%d %d", mesh.el_tags[e], np);
                for (int n = 0; n < np; ++n) {
                    size_t i = (size_t)e * np + n;
                    if (v == 0) std::fprintf(f, " %.17g", fr.u[i]);
                    else if (v == 1) std::fprintf(f, " %.17g", fr.u[i] / (cfg.c0 * cfg.c0));
                    else
                        std::fprintf(f, " %.17g %.17g %.17g", fr.u[ndof + i], fr.u[2 * ndof + i], fr.u[3 * ndof + i]);
                }
                std::fprintf(f, "\n");
            }
            std::fprintf(f, "$EndElementNodeData\n");
        }
    }
    std::fclose(f);
    return true;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) return E2BIG;
    const std::string msh = argv[1], conf = argv[2];
    dg::RawMesh mesh;
    std::string err = dg::read_msh(msh, mesh);
    if (!err.empty()) {
        std::fprintf(stderr, "Error   : %s\n", err.c_str());
        return EXIT_FAILURE;
    }
    dg::Config cfg;
    err = dg::parse_config(conf, mesh, cfg);
    if (!err.empty()) {
        std::fprintf(stderr, "Error   : %s\n", err.c_str());
        return EXIT_FAILURE;
    }
    for (auto &w : cfg.warnings) log(w);
    std::remove(cfg.saveFile.c_str());
    log("Config loaded : " + conf);
    std::vector<std::pair<int, bool>> bcs(cfg.physBCs.begin(), cfg.physBCs.end());
    dg::Precomp pre;
    err = dg::precompute(mesh, bcs, pre);
    if (!err.empty()) {
        std::fprintf(stderr, "Error   : %s\n", err.c_str());
        return EXIT_FAILURE;
    }
    log("Number of Elements : " + std::to_string(pre.K));
    log("Element dimension : " + std::to_string(pre.dim));
    log("Element Order : " + std::to_string(pre.order));
    log("Number of Faces : " + std::to_string(pre.F));
    if (pre.ncurved > 0)
        log("Curved elements : " + std::to_string(pre.ncurved) + " (per-point geometry on " +
            std::to_string(pre.ng) + " element / " + std::to_string(pre.ngf) + " face points)");
    const size_t ndof = (size_t)pre.K * pre.np;

    // initial conditions (dgalerkin.cpp:37-50)
    std::vector<double> u(4 * ndof, 0.0);
    for (auto &ic : cfg.initConditions)
        for (size_t n = 0; n < ndof; ++n) {
            const double *c = &pre.dof_xyz[n * 3];
            u[n] += ic[5] * std::exp(-((c[0] - ic[1]) * (c[0] - ic[1]) + (c[1] - ic[2]) * (c[1] - ic[2]) +
                                       (c[2] - ic[3]) * (c[2] - ic[3])) /
                                     ic[4]);
        }

    // integrator dispatch (dgalerkin.cpp:55-58): "Euler1" (the default) or
    // "Runge-Kutta"; any other name runs no solver and writes no views
    int (*run_steps)(dg_ctx *, double *, double, int) = nullptr;
    if (cfg.timeIntMethod == "Euler1") run_steps = dg_euler_steps;
    else if (cfg.timeIntMethod == "Runge-Kutta") run_steps = dg_rk4_steps;
    else {
        log("Solver '" + cfg.timeIntMethod + "' is not a known method: nothing to run");
        return EXIT_SUCCESS;
    }
    dg_mesh_desc desc;
    dg::fill_desc(pre, desc);
    dg_phys_desc phys;
    phys.c0 = cfg.c0; phys.rho0 = cfg.rho0;
    for (int k = 0; k < 3; ++k) phys.v0[k] = cfg.v0[k];
    dg_opts opts;
    dg_default_opts(&opts);
    opts.precision = cfg.precision == "fp32"     ? DG_PREC_FP32
                     : cfg.precision == "mixed"  ? DG_PREC_MIXED
                     : cfg.precision == "tf32x3" ? DG_PREC_TF32X3
                                                 : DG_PREC_FP64;
    opts.flux_sign = cfg.fluxSign == "upwind" ? DG_FLUX_UPWIND : DG_FLUX_REFERENCE;
    dg_ctx *ctx = nullptr;
    if (dg_create(&desc, &phys, &opts, &ctx) != DG_OK) {
        std::fprintf(stderr, "Error   : %s\n", dg_last_error());
        return EXIT_FAILURE;
    }
    const double *uq[4] = {&u[0], &u[ndof], &u[2 * ndof], &u[3 * ndof]};
    int rc = dg_set_state(ctx, uq);
    // sources (solver.cpp:197-210)
    if (rc == DG_OK && !cfg.sources.empty()) {
        std::vector<int> off(1, 0), idx;
        std::vector<double> par;
        for (auto &s : cfg.sources) {
            for (size_t n = 0; n < ndof; ++n) {
                const double *c = &pre.dof_xyz[n * 3];
                if (std::pow(c[0] - s[1], 2) + std::pow(c[1] - s[2], 2) + std::pow(c[2] - s[3], 2) < std::pow(s[4], 2))
                    idx.push_back((int)n);
            }
            off.push_back((int)idx.size());
            par.insert(par.end(), {s[5], s[6], s[7], s[8]});
        }
        if (idx.empty()) idx.push_back(0);
        rc = dg_set_sources(ctx, (int)cfg.sources.size(), off.data(), idx.data(), par.data());
    }
    // time loop (solver.cpp:216-286, and 107-154 for Euler1): saves happen
    // before the step at t
    std::vector<Frame> frames;
    auto start = std::chrono::system_clock::now();
    double t_run = cfg.timeStart;  // time at the start of the pending steps
    int pending = 0;
    double t = cfg.timeStart, step = 0, tDisplay = 0;
    for (; rc == DG_OK && t <= cfg.timeEnd; t += cfg.timeStep, tDisplay += cfg.timeStep, ++step) {
        if (tDisplay >= cfg.timeRate || step == 0) {
            tDisplay = 0;
            if (pending) {
                rc = run_steps(ctx, &t_run, cfg.timeStep, pending);
                pending = 0;
                if (rc != DG_OK) break;
            }
            // the copy-out overlaps the steps that follow (the reference
            // copies the state into its views here, solver.cpp:226-235)
            frames.emplace_back();
            Frame &fr = frames.back();
            fr.t = t;
            fr.step = (int)step;
            fr.u = static_cast<double *>(dg_host_alloc(4 * ndof * sizeof(double)));
            if (!fr.u) {
                fr.own.resize(4 * ndof);
                fr.u = fr.own.data();
            }
            rc = dg_get_state_async(ctx, fr.u, &fr.ticket);
            if (rc != DG_OK) break;
            auto el = std::chrono::duration_cast<std::chrono::seconds>(std::chrono::system_clock::now() - start);
            log("[" + std::to_string(t) + "/" + std::to_string(cfg.timeEnd) + "s] Step number : " +
                std::to_string((int)step) + ", Elapsed time: " + std::to_string(el.count()) + "s");
            t_run = t;
        }
        ++pending;
    }
    if (rc == DG_OK && pending) rc = run_steps(ctx, &t_run, cfg.timeStep, pending);
    for (Frame &fr : frames)
        if (rc == DG_OK && fr.ticket >= 0) rc = dg_wait_state(ctx, fr.ticket);
    auto release = [&]() {
        for (Frame &fr : frames)
            if (fr.own.empty()) dg_host_free(fr.u);
    };
    if (rc != DG_OK) {
        std::fprintf(stderr, "Error   : %s\n", dg_last_error());
        dg_destroy(ctx);  // waits for copies still in flight
        release();
        return EXIT_FAILURE;
    }
    dg_destroy(ctx);
    const bool ok = write_views(cfg.saveFile, mesh, pre, cfg, frames);
    release();
    if (!ok) return EXIT_FAILURE;
    log("Views written to " + cfg.saveFile);
    return EXIT_SUCCESS;
}
