"""Benchmark of the DG acoustic RK4 right-hand side on one GB300.

Workload (the configuration the metric is quoted on): unit cube as a 40^3 hex
grid, each hex split into 6 tetrahedra (384,000 tets), order 3 (Np = 20),
linearised Euler with uniform mean flow Mach 0.3 along x (c0 = 340,
rho0 = 1.225), absorbing boundaries, Gaussian pressure pulse sigma = 0.05 at
a seeded interior point, dt from CFL 0.5.  Four evolved fields (p, vx, vy,
vz); density is p/c0^2 at output.  A step is one classical RK4 time step
(four fused stage launches).  The chosen form (--form, default "mixed") keeps
FP32 stage data, the state as an FP32 pair, and runs the volume + lift
contraction on the tcgen05 tensor cores with exact fixed-point accumulation;
the plain FP64 form and the FP32 CUDA-core form are measured beside it, and
every form's error against FP64 is measured after the configuration's 2000
steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  --impl reference times the reference's CPU
algorithm (the oracle restatement) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "dgfem-acoustic_gb300"
sys.path.insert(0, str(PKG))

METRIC = "DOF-stage updates/s, chosen vs plain DG on one GB300 at rel-L2<=1e-5 vs FP64"
UNIT = "DOF-stage/s"
C0, RHO0 = 340.0, 1.225
MACH = 0.3
SIGMA = 0.05
SEED = 2026
NCELL = 40
ORDER = 3
FLUX = "upwind"
WORKLOAD = (f"unit cube {NCELL}^3 hexes x 6 tets ({NCELL ** 3 * 6} tets), order {ORDER} (Np=20), LEE with "
            f"uniform mean flow Mach {MACH} along x, absorbing boundaries, Gaussian pulse sigma {SIGMA} at a "
            f"seeded interior point, dt from CFL 0.5, classical RK4")
FALLBACK_HBM_GBS = 6800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------- setup
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def ensure_built():
    import dgcuda

    if not dgcuda.LIB_PATH.exists():
        sys.path.insert(0, str(ROOT))
        import __graft_entry__

        __graft_entry__.build()


def workload(n=NCELL, order=ORDER):
    import dgcuda as D

    mesh = D.Mesh.box_tet(n, n, n, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), order=order, side_names=("Absorbing",) * 6)
    pre = D.Precomp(mesh)
    v0 = (MACH * C0, 0.0, 0.0)
    dt = D.cfl_dt(pre, C0, v0, 0.5)
    centre = np.random.default_rng(SEED).uniform(0.3, 0.7, 3)
    ic = (0.0, *centre, 2 * SIGMA ** 2, 1.0)
    return mesh, pre, v0, dt, ic


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(name: str):
    """Per-launch DRAM bytes recorded from an ncu capture in profiles/."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, interval_ms: int = 100):
        self.device, self.interval = device, interval_ms
        self.proc, self.lines = None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.lines:
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ byte model
def stage_bytes(pre, real_bytes: int, pair_state: bool = False, geo_bytes: int = 8) -> list[float]:
    """Algorithmic HBM bytes of each fused stage launch (unique bytes: state
    reads/writes, geometry once; neighbour traces are L2 re-reads).
    Stage 1 reads u, writes acc and w; stages 2-3 read w, u, acc and write
    acc, w; stage 4 reads w, u, acc and writes u.  With the state kept as an
    FP32 pair (mixed form) every read of u also reads its low part and stage 4
    writes both.  geo_bytes: size of an inverse-Jacobian entry (FP64 in the
    FP64 form, FP32 in the others)."""
    nq = pre.dim + 1
    n = pre.ndof * nq
    geo = pre.num_el * (pre.dim * pre.dim * geo_bytes + pre.nf * 4 * real_bytes + pre.nf * 8)
    words = (4, 6, 6, 6) if pair_state else (3, 5, 5, 4)
    return [n * real_bytes * k + geo for k in words]


# ------------------------------------------------------------------ CPU (oracle)
def oracle_box(n: int, order: int = ORDER):
    """The workload's mesh built for the oracle alone (NumPy and the oracle's
    own reference lattice; the product library is not loaded): the unit cube
    as n^3 hexes, each split into the 6 tetrahedra along the paths of the
    axis permutations (the box generator's split and orientation), order
    `order` nodes in gmsh order, node tags from the global node lattice, no
    physical groups (every boundary face absorbing, the reference's default
    BC, Mesh.cpp:364-384).  Returns the raw mesh dict the oracle reads, the
    node coordinates of every element [K][np][3] and the CFL-0.5 time step."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O

    R = np.rint(O.reference_element(3, order)["nodes"] * order).astype(np.int64)  # [np][3]
    tets = []
    for pm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        x = [0, 0, 0]
        V = [list(x)]
        for ax in pm:
            x[ax] += 1
            V.append(list(x))
        V = np.array(V, dtype=np.int64)
        if np.linalg.det((V[1:] - V[0]).astype(float)) < 0:
            V[[1, 2]] = V[[2, 1]]
        tets.append(V)
    T = np.array(tets)  # [6][4][3]
    off = (order * T[:, 0, None, :] + R[None, :, 0, None] * (T[:, 1] - T[:, 0])[:, None, :] +
           R[None, :, 1, None] * (T[:, 2] - T[:, 0])[:, None, :] + R[None, :, 2, None] * (T[:, 3] - T[:, 0])[:, None, :])
    kk, jj, ii = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    cell = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.int64) * order
    L = cell[:, None, None, :] + off[None]  # [cells][6][np][3]
    n1 = n * order + 1
    key = L[..., 0] + n1 * (L[..., 1] + n1 * L[..., 2])
    np_ = R.shape[0]
    el_nodes = (key.reshape(-1, np_) + 1).astype(np.int32)
    g = np.arange(n1, dtype=np.float64) / (n * order)
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)
    K = el_nodes.shape[0]
    raw = {"dim": 3, "order": order, "np": np_, "node_tags": np.arange(1, n1 ** 3 + 1, dtype=np.int32), "xyz": xyz,
           "el_tags": np.arange(1, K + 1, dtype=np.int32), "el_nodes": el_nodes,
           "phys_dim": np.zeros(0, np.int32), "phys_tag": np.zeros(0, np.int32),
           "phys_offsets": np.zeros(1, np.int32), "phys_nodes": np.zeros(0, np.int32)}
    X = xyz[el_nodes - 1]  # [K][np][3]
    v = X[:, :4, :]
    a, b, c = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]
    vol = np.abs(np.einsum("ij,ij->i", a, np.cross(b, c))) / 6
    surf = sum(0.5 * np.linalg.norm(np.cross(v[:, j] - v[:, i], v[:, k] - v[:, i]), axis=1)
               for i, j, k in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)))
    r_in = float(np.min(3 * vol / surf))
    dt = 0.5 * 2 * r_in / ((2 * order + 1) * (C0 + MACH * C0))
    return raw, X, dt


def oracle_workload(n: int = NCELL):
    """Mesh, initial state (the reference's Gaussian pulse, dgalerkin.cpp:37-50)
    and time step of the workload at n^3 cells, for the oracle alone."""
    raw, X, dt = oracle_box(n)
    centre = np.random.default_rng(SEED).uniform(0.3, 0.7, 3)
    u0 = np.zeros((4, X.shape[0] * X.shape[1]))
    r2 = ((X.reshape(-1, 3) - centre) ** 2).sum(axis=1)
    u0[0] = 1.0 * np.exp(-r2 / (2 * SIGMA ** 2))
    return raw, u0, dt, (MACH * C0, 0.0, 0.0)


def oracle_sample_rate(n: int, steps: int, threads: int, dedup: bool = False):
    """Faithful CPU restatement timed on an n^3 x 6 sample of the workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O

    raw, u0, dt, v0 = oracle_workload(n)
    orc = O.Oracle(raw, dt, C0, RHO0, v0=v0, upwind=(FLUX == "upwind"), num_threads=threads)
    orc.set_state(u0)
    _, sec = orc.run(0.0, steps, dedup=dedup)
    num_el = raw["el_nodes"].shape[0]
    dofstage = num_el * raw["np"] * 4 * 4 * steps
    return dofstage / sec, sec, num_el


def cpu_baseline(target_s: float = 15.0):
    threads = os.cpu_count() or 1
    # calibrate on a small sample, then size the sample for ~target_s
    rate_small, sec_small, _ = oracle_sample_rate(4, 1, threads)
    n = 4
    for cand in (6, 8, 10, 12, 16):
        est = sec_small * (cand / 4) ** 3
        if est * 3 <= target_s:
            n = cand
    _, sec1, _ = oracle_sample_rate(n, 1, threads)
    steps = max(1, min(40, int(target_s / max(sec1, 1e-3))))
    rate, sec, num_el = oracle_sample_rate(n, steps, threads)
    rate_dedup, _, _ = oracle_sample_rate(n, max(1, steps // 2), threads, dedup=True)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n}^3 x 6 = {num_el} tets of the same workload (order 3, Mach 0.3, absorbing), "
                      f"{steps} RK4 steps, {sec:.1f} s, faithful nested-OpenMP face loop",
            "dedup_face_loop_value": rate_dedup}


def workload_config(num_el: int, ndof: int, nq: int, dt: float, world: int, cells: int = NCELL) -> dict:
    """The `config` object of both arms' JSON lines (same workload, same keys)."""
    return {"workload": WORKLOAD if cells == NCELL else WORKLOAD + f" (profiling case: {cells}^3 cells)",
            "tets": num_el, "dofs_per_field": ndof, "fields": nq, "dt": float(f"{dt:.9e}"), "flux_sign": FLUX,
            "l2": "inputs larger than L2 (FP32 state 4 x %.0f MB)" % (ndof * nq * 4 / 1e6),
            "parallelism": "replicas" if world > 1 else "single GPU"}


REFERENCE_SAMPLE_REASON = (
    "one RK4 step of the full 384,000-tet workload takes about 25 s in the faithful restatement on the GPU "
    "host's 16 cores (its face loop runs once per OpenMP thread, as in the reference), so --steps 20 --warmup 5 "
    "would take over 10 minutes; each step therefore runs an n^3 x 6 sample of the same workload, the largest "
    "that keeps the run within --reference-seconds, and the rate is per DOF-stage")


def reference_arm(args, world, rank, pg):
    """The reference's CPU algorithm (the faithful oracle restatement; the
    reference itself cannot be built here) on the host cores.  Only the
    oracle library is loaded: mesh, initial state and time step come from
    oracle_box/oracle_workload."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    total = args.steps + args.warmup
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O

    full = args.reference_full
    if full:
        n = NCELL
    else:
        # per-step sample sized so the whole run stays within --reference-seconds
        _, sec4, _ = oracle_sample_rate(4, 1, threads)
        n = 2
        for cand in (3, 4, 6, 8, 10, 12, 16, 20):
            if sec4 * (cand / 4) ** 3 * total <= args.reference_seconds:
                n = cand
    raw, u0, dt, v0 = oracle_workload(n)
    t_setup = time.time()
    orc = O.Oracle(raw, dt, C0, RHO0, v0=v0, upwind=(FLUX == "upwind"), num_threads=threads)
    orc.set_state(u0)
    setup_s = time.time() - t_setup
    t = 0.0
    if args.warmup:
        t, _ = orc.run(t, args.warmup)
    t, sec = orc.run(t, args.steps)
    num_el = raw["el_nodes"].shape[0]
    ndof = num_el * raw["np"]
    value = ndof * 4 * 4 * args.steps / sec
    # the config of the GPU arm: the full workload.  Its cells are the
    # sample's scaled by n / NCELL (congruent tetrahedra), so is its time step.
    dt_full = dt * n / NCELL
    sample = (f"full workload, {num_el} tets" if full else
              f"{n}^3 x 6 = {num_el} tets of the same workload per step") + \
        f", {args.steps} timed RK4 steps, {sec:.1f} s (setup {setup_s:.1f} s, not timed)"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "form": "reference CPU algorithm (faithful C++/OpenMP restatement of Mesh.cpp/solver.cpp)",
            "config": workload_config(NCELL ** 3 * 6, NCELL ** 3 * 6 * 20, 4, dt_full, world),
            "sample": sample, "sample_reason": None if full else REFERENCE_SAMPLE_REASON,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
FORMS = {
    "mixed": ("FP32 stage data, state kept as an FP32 pair, volume + lift contraction on the tcgen05 tensor "
              "cores with BF16 fixed-point slices and exact FP32 accumulation, FP32 geometry factors",
              "f32+bf16x4 (exact accumulation)", "mixed_stage_kernel<3,3> (tcgen05 kind::f16, A in TMEM)"),
    "fp32": ("FP32 state, flux and geometry factors, fused stage kernel on CUDA cores", "f32",
             "stage_kernel<3,3,float>"),
    "fp64": ("FP64 throughout, fused stage kernel on CUDA cores", "f64", "stage_kernel<3,3,double>"),
    "tf32x3": ("FP32 stage data, state kept as an FP32 pair, volume + lift contraction on the tcgen05 tensor "
               "cores by 3xTF32 split products (a_hi b_hi + a_hi b_lo + a_lo b_hi) with FP32 accumulation",
               "f32+tf32x3", "mixed_stage_kernel<3,3,...,kTcTf32x3> (tcgen05 kind::tf32, A in TMEM)"),
}


def roofline_for(sol, pre, form, t, dt, nprof):
    _, prof = sol.profile_steps(t, dt, nprof)
    real = 8 if form == "fp64" else 4
    sb = stage_bytes(pre, real, pair_state=(form in ("mixed", "tf32x3")), geo_bytes=real)
    avg_ms = [prof["stage_ms"][s] / max(prof["stage_launches"][s], 1) for s in range(4)]
    achieved = sum(sb) / (sum(avg_ms) * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic(f"stage_kernel_cube40_p3_{form}.md")
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": peak_kind, "algorithmic_bytes_per_launch": sum(sb) / 4,
            "stage_ms": avg_ms, "kernel": FORMS[form][2]}


def timed_form(D, pre, form, u0, dt, v0, local, steps, warmup):
    sol = D.Solver(pre, C0, RHO0, v0, precision=form, flux=FLUX, device=local)
    sol.set_state(u0)
    t = sol.rk4_steps(0.0, dt, warmup)
    t, ms = sol.rk4_steps_timed(t, dt, steps)
    return sol, t, ms


def ours_arm(args, world, rank, local, pg):
    import dgcuda as D

    ensure_built()
    t_setup = time.time()
    mesh, pre, v0, dt, ic = workload(args.cells)
    u0 = pre.initial_state([ic])
    log(f"[bench] rank {rank}: mesh {pre.num_el} tets, {pre.ndof} DOF/field, dt {dt:.3e}, setup "
        f"{time.time() - t_setup:.1f}s")
    nq = pre.dim + 1
    dof_stage_per_step = pre.ndof * nq * 4
    form = args.form

    sol = D.Solver(pre, C0, RHO0, v0, precision=form, flux=FLUX, device=local)
    sol.set_state(u0)
    t = sol.rk4_steps(0.0, dt, args.warmup)

    # timed region: K steps, CUDA events on the solver stream, graph chunks
    barrier(pg)
    sol.synchronize()
    with ClockSampler(local) as clk:
        t, ms = sol.rk4_steps_timed(t, dt, args.steps)
    sol.synchronize()
    barrier(pg)
    ms_max = allreduce_max(pg, ms)
    units = allreduce_sum(pg, dof_stage_per_step * args.steps)
    value = units / (ms_max * 1e-3)
    e, _, bad = sol.monitors()
    roofline = roofline_for(sol, pre, form, t, dt, min(args.steps, 100))

    # end to end: every step's input copied in from pinned host memory, one
    # step, and the step's result copied out to pinned host memory, through
    # the C ABI.  The copy-in is dg_stage_state (started before the previous
    # step runs, so it crosses the host link meanwhile) and dg_commit_state;
    # the copy-out is dg_get_state_async (the save-step API) on a side stream
    # while the next step's input goes in and the next step computes; the
    # run waits for every frame before the clock stops.
    n_e2e = 0 if args.no_e2e else min(args.steps, 200)
    nbytes = 4 * pre.ndof * 8
    e2e_value = e2e_sync_value = None
    if n_e2e:
        uin = D.pinned_array((4, pre.ndof))
        outs = [D.pinned_array((4, pre.ndof)), D.pinned_array((4, pre.ndof))]
        uin[:] = u0
        barrier(pg)
        sol.synchronize()
        w0 = time.perf_counter()
        te = 0.0
        tickets = []
        tk = sol.stage_state(uin)
        for k in range(n_e2e):
            sol.commit_state(tk)
            if k + 1 < n_e2e:
                tk = sol.stage_state(uin)  # the next step's input, while this step runs
            te = sol.rk4_steps(te, dt, 1)
            tickets.append(sol.get_state_async(outs[k % 2]))
        for tk in tickets[-2:]:
            sol.wait_state(tk)  # earlier frames were waited for when their slot was reused
        sol.synchronize()
        w1 = time.perf_counter()
        barrier(pg)
        e2e_value = allreduce_sum(pg, dof_stage_per_step * n_e2e) / allreduce_max(pg, w1 - w0)
        # the blocking protocol beside it (dg_set_state before and dg_get_state
        # after each step, each waited for)
        n_sync = min(n_e2e, 50)
        sol.synchronize()
        w0 = time.perf_counter()
        te = 0.0
        for _ in range(n_sync):
            sol.set_state(uin)
            te = sol.rk4_steps(te, dt, 1)
            sol.get_state(outs[0])
        sol.synchronize()
        w1 = time.perf_counter()
        e2e_sync_value = allreduce_sum(pg, dof_stage_per_step * n_sync) / allreduce_max(pg, w1 - w0)
    sol.close()

    # the other forms on the same workload, and the accuracy of every form
    # against the FP64 form after the configuration's steps
    others = {}
    if not args.no_plain:
        for f2 in ("fp64", "fp32", "mixed", "tf32x3"):
            if f2 == form:
                continue
            nsteps = max(5, min(args.steps, 40 if f2 == "fp64" else 400))
            s2, t2, ms2 = timed_form(D, pre, f2, u0, dt, v0, local, nsteps, 3)
            others[f2] = {"value": dof_stage_per_step * nsteps / (ms2 * 1e-3), "unit": UNIT,
                          "ms_per_step": ms2 / nsteps, "form": FORMS[f2][0],
                          "roofline": roofline_for(s2, pre, f2, t2, dt, 5 if f2 == "fp64" else 40)}
            s2.close()
    acc = None
    if args.accuracy_steps > 0 and not args.no_plain:
        acc = accuracy_all(D, pre, u0, dt, v0, args, local, nq)
    if "fp64" in others:
        others["fp64"]["chosen_over_this"] = value / others["fp64"]["value"]

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.cpu_seconds)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": FORMS[form][1], "data": "synthetic",
        "form": FORMS[form][0],
        "config": workload_config(pre.num_el, pre.ndof, nq, dt, world, args.cells),
        "accuracy": acc,
        "plain_fp64": others.get("fp64"),
        "other_forms": {k: v for k, v in others.items() if k != "fp64"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": n_e2e,
                "how": "per step: dg_stage_state of that step's input from pinned host (side-stream copy "
                       "started before the previous step runs) and dg_commit_state, dg_rk4_steps(1), "
                       "dg_get_state_async into pinned host (side-stream copy overlapping the next step); every "
                       "frame waited for before the clock stops",
                "blocking_copy_out_value": e2e_sync_value,
                "blocking_how": "per step: dg_set_state, dg_rk4_steps(1), dg_get_state, each waited for"},
        "clocks": clk.summary(),
        "gpu_launches": 4 * args.steps,
        "monitors": {"energy": e, "nonfinite": bad},
    }
    if world == 1 and not args.no_batched:
        line["batched"] = batched_section(D, args, local)
    if world == 1 and not args.no_uneven:
        line["uneven_batch"] = uneven_section(D, args, local)
    if world == 1 and not args.no_parareal:
        line["learned_parareal"] = parareal_section(D, args, local)
    if world == 1 and not args.no_curved:
        line["curved"] = curved_section(D, args, local)
    print(json.dumps(line), flush=True)


def batched_section(D, args, local):
    """Multi-source batch: unit cube 40^3 x 6 tets, order 4, 64 Gaussian
    sources (one per batch member) and 16 receivers, zero initial state.  The
    mixed form and the FP64 form each run the whole batch in one launch per
    stage; accuracy: the first members of the mixed batch against the FP64
    batch after acc_steps steps (state and receiver traces)."""
    from dgcuda import workloads as W

    t0 = time.time()
    mesh, pre, dt, srcs, recs = W.multi_source(n=args.batched_cells, order=4, nsrc=args.batched_sources, seed=SEED)
    log(f"[bench] batched: {pre.num_el} tets x {args.batched_sources} sources, {pre.ndof} DOF/field, "
        f"setup {time.time() - t0:.1f}s")
    zero = np.zeros((4, pre.ndof))
    units_per_step = pre.ndof * 4 * 4 * args.batched_sources
    out = {"workload": f"unit cube {args.batched_cells}^3 hexes x 6 tets ({pre.num_el} tets), order 4 (Np=35), "
                       f"{args.batched_sources} Gaussian sources (sigma 0.03, f in [2,8], positions in [0.1,0.9]^3, "
                       f"one per batch member), 16 receivers, zero initial state, absorbing walls",
           "unit": UNIT, "dofs_per_field": pre.ndof, "members": args.batched_sources, "dt": dt}
    for form, steps in (("mixed", args.batched_steps), ("tf32x3", args.batched_steps),
                        ("fp64", max(2, args.batched_steps // 5))):
        s = D.Solver(pre, C0, RHO0, (0.0, 0.0, 0.0), precision=form, flux=FLUX, device=local,
                     nbatch=args.batched_sources)
        s.set_state(zero)
        s.set_batch_sources(srcs)
        s.set_receivers(recs, steps + 3)
        t = s.rk4_steps(0.0, dt, 3)
        with ClockSampler(local) as clk:
            t, ms = s.rk4_steps_timed(t, dt, steps)
        out[form] = {"value": units_per_step * steps / (ms * 1e-3), "steps": steps, "ms_per_step": ms / steps,
                     "clocks": clk.summary()}
        s.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["tf32x3_over_fp64"] = out["tf32x3"]["value"] / out["fp64"]["value"]
    out["accuracy"] = batched_accuracy(D, pre, dt, srcs, recs, min(4, args.batched_sources),
                                       args.batched_acc_steps, local)
    # the batch's chosen form: the fastest tensor-core form whose measured
    # error against the FP64 batch meets 1e-5
    ok = [f for f in ("mixed", "tf32x3") if out["accuracy"][f]["meets_1e-5"]]
    if ok:
        best = max(ok, key=lambda f: out[f]["value"])
        out["chosen"] = {"form": best, "value": out[best]["value"], "over_fp64": out[best]["value"] / out["fp64"]["value"],
                         "rel_l2_vs_fp64": out["accuracy"][best]["state_rel_l2_vs_fp64_max"]}
    return out


def batched_accuracy_section(D, args, local):
    """Accuracy of the multi-source batch as configured: every one of the 64
    members after 1000 steps against the FP64 batch.  The FP64 batch of the
    40^3 order-4 mesh would need ~1.8 h for 1000 steps (2.2 G DOF-stage/s),
    so this case keeps the configuration's sources, receivers, order and step
    count on a coarser cube (--batched-acc-cells, default 12^3 x 6 tets)."""
    from dgcuda import workloads as W

    t0 = time.time()
    mesh, pre, dt, srcs, recs = W.multi_source(n=args.batched_acc_cells, order=4, nsrc=args.batched_sources,
                                               seed=SEED)
    log(f"[bench] batched accuracy: {pre.num_el} tets x {args.batched_sources} sources, setup {time.time() - t0:.1f}s")
    t0 = time.time()
    res = batched_accuracy(D, pre, dt, srcs, recs, args.batched_sources, args.batched_acc_all_steps, local)
    res["workload"] = (f"unit cube {args.batched_acc_cells}^3 hexes x 6 tets ({pre.num_el} tets), order 4, "
                       f"{args.batched_sources} Gaussian sources (sigma 0.03, f in [2,8], positions in [0.1,0.9]^3), "
                       f"16 receivers, zero initial state, absorbing walls")
    res["seconds"] = time.time() - t0
    return res


def batched_accuracy(D, pre, dt, srcs, recs, nacc, steps, local):
    """Members 0..nacc-1 of the tensor-core batches against the FP64 batch
    after `steps` steps (same sources): the largest relative L2 over members
    and fields (FP64 error monitor on the device) and the receiver traces."""
    zero = np.zeros((4, pre.ndof))
    sols, traces = {}, {}
    for form in ("fp64", "mixed", "tf32x3"):
        s = D.Solver(pre, C0, RHO0, (0.0, 0.0, 0.0), precision=form, flux=FLUX, device=local, nbatch=nacc)
        s.set_state(zero)
        s.set_batch_sources([x for x in srcs if x[0] < nacc])
        s.set_receivers(recs, steps)
        s.rk4_steps(0.0, dt, steps)
        traces[form] = s.traces()
        sols[form] = s
    res = {"members": nacc, "steps": steps}
    for form in ("mixed", "tf32x3"):
        err = max(max(sols[form].error_vs(sols["fp64"], member=m, ref_member=m)[0]) for m in range(nacc))
        terr = float(np.linalg.norm(traces[form] - traces["fp64"]) / np.linalg.norm(traces["fp64"]))
        res[form] = {"state_rel_l2_vs_fp64_max": float(err), "receiver_traces_rel_l2_vs_fp64": terr,
                     "meets_1e-5": bool(err <= 1e-5)}
    for s in sols.values():
        s.close()
    return res


def uneven_section(D, args, local):
    """Uneven batch: 32 seeded boxes (5k-300k tets, order 2-5, one Gaussian
    source each, mixed wall types) in FP32, one persistent launch per stage
    for all meshes; tile configuration chosen by the autotuner; compared with
    the same meshes stepped one context at a time."""
    from dgcuda import workloads as W

    t0 = time.time()
    meshes, pres, phys, dts, srcs = W.uneven(nmesh=args.uneven_meshes, seed=SEED)
    tets = [p.num_el for p in pres]
    orders = [p.order for p in pres]
    log(f"[bench] uneven: {len(pres)} meshes, {sum(tets)} tets, setup {time.time() - t0:.1f}s")
    units_per_step = sum(p.ndof for p in pres) * 4 * 4
    ms_ = D.MultiSolver(pres, phys, precision="fp32", flux=FLUX, device=local)
    for i, p in enumerate(pres):
        ms_.set_state(i, np.zeros((4, p.ndof)))
    ms_.set_sources(srcs)
    chosen, cand = ms_.autotune(dts, trial_steps=5)
    t = ms_.rk4_steps(np.zeros(len(pres)), dts, 3)
    with ClockSampler(local) as clk:
        t, ms = ms_.rk4_steps_timed(t, dts, args.uneven_steps)
    info = ms_.info()
    names = [f"one launch, {b}-thread CTAs" if b else "one launch per order" for b in info["block_threads"]]
    ms_.close()
    # the same meshes, one single-mesh context each, stepped one after the other
    nsep = max(3, args.uneven_steps // 10)
    sep_ms = 0.0
    for i, p in enumerate(pres):
        s = D.Solver(p, *phys[i], precision="fp32", flux=FLUX, device=local)
        s.set_state(np.zeros((4, p.ndof)))
        s.set_batch_sources([(0, *srcs[i][1:])])
        tt = s.rk4_steps(0.0, dts[i], 3)
        _, m1 = s.rk4_steps_timed(tt, dts[i], nsep)
        sep_ms += m1 / nsep
        s.close()
    value = units_per_step * args.uneven_steps / (ms * 1e-3)
    return {"workload": f"{len(pres)} seeded boxes, side lengths in [0.5,3], h 0.025 coarsened to keep "
                       f"{min(tets)}-{max(tets)} tets per mesh ({sum(tets)} tets), orders {sorted(set(orders))}, "
                       "one Gaussian source each, mixed reflecting/absorbing sides, FP32",
            "unit": UNIT, "value": value, "steps": args.uneven_steps, "ms_per_step": ms / args.uneven_steps,
            "tile_config": {"chosen": names[chosen],
                            "candidates_ms_per_step": dict(zip(names, cand))},
            "separate_contexts_ms_per_step": sep_ms,
            "one_launch_over_separate": sep_ms / (ms / args.uneven_steps),
            "clocks": clk.summary()}


def curved_flops(pre, info) -> float:
    """Algorithmic flops of one curved element in one stage launch: flux at
    the element points (interpolation, flux, w detJ J^-T), stiffness
    contraction, traces of both sides at the face points, face flux,
    projection on the face basis, inverse mass."""
    d, np_, nq, nf, nfp = pre.dim, pre.np, pre.dim + 1, pre.nf, pre.nfp
    ng, ngf = info["curved_points"], info["curved_face_points"]
    fma = (ng * np_ * nq + ng * (d * nq + d * d * nq) + d * ng * np_ * nq + 2 * nf * ngf * nfp * nq + nf * ngf * 20
           + nf * nfp * ngf * nq + np_ * np_ * nq)
    return 2.0 * fma


def curved_section(D, args, local):
    """Curved (isoparametric) elements: unit cube n^3 x 6 tets, order 3, its
    nodes moved by a smooth map that curves every element ("full") or the
    elements with x > 1/2 ("half"), against the straight cube; FP64, FP32 and
    mixed contexts; RK4.  Per variant the whole-step rate, and the per-point
    kernel's device time per launch (CUDA events) with its FP64/FP32
    arithmetic rate and HBM bytes rate.  CPU baseline: the oracle (per-point
    form for every element, as the reference) on a smaller fully curved cube."""
    from dgcuda import workloads as W

    n, steps = args.curved_cells, args.curved_steps
    out = {"workload": f"unit cube {n}^3 x 6 tets, order 3, absorbing walls, nodes moved by a smooth map "
                       "(amplitude 0.02) curving all ('full') or half ('half') of the elements; RK4",
           "unit": UNIT, "variants": []}
    for kind in ("none", "half", "full"):
        mesh, pre = W.curved_cube(n, 3, kind)
        dt = D.cfl_dt(pre, C0)
        u0 = pre.initial_state([(0, 0.5, 0.5, 0.5, 2 * SIGMA ** 2, 1.0)])
        units = pre.ndof * 4 * 4
        for prec in ("fp64", "fp32", "mixed"):
            s = D.Solver(pre, C0, RHO0, precision=prec, flux=FLUX, device=local)
            s.set_state(u0)
            t = s.rk4_steps(0.0, dt, args.warmup)
            t, ms = s.rk4_steps_timed(t, dt, steps)
            _, kt = s.profile_steps(t, dt, 2)
            info = s.info()
            v = {"kind": kind, "form": prec, "tets": pre.num_el, "curved": info["curved"],
                 "value": units * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                 "affine_kernel_ms_per_launch": sum(kt["stage_ms"]) / max(sum(kt["stage_launches"]), 1)}
            if kt["curved_launches"]:
                cms = kt["curved_ms"] / kt["curved_launches"]
                rb = 8 if prec == "fp64" else 4
                # the mixed form also reads the state's low part and writes it in the last stage
                C, ng, ngf = info["curved"], info["curved_points"], info["curved_face_points"]
                # per curved element: inverse mass, metric, face data (context precision), state
                # (stage input, u, acc read; acc, next input written: about 5 values per DOF)
                nbytes = C * (rb * (pre.np ** 2 + ng * 9 + pre.nf * ngf * 4) + 5 * rb * pre.np * 4)
                fl = C * curved_flops(pre, info)
                v.update({"curved_kernel_ms_per_launch": cms,
                          "curved_kernel_tflops": fl / (cms * 1e-3) / 1e12,
                          "curved_kernel_gbs": nbytes / (cms * 1e-3) / 1e9,
                          "curved_kernel_dof_stage_per_s": C * pre.np * 4 / (cms * 1e-3)})
            out["variants"].append(v)
            s.close()
        log(f"[bench] curved {kind}: {pre.num_curved}/{pre.num_el} curved, "
            + ", ".join(f"{x['form']} {x['value'] / 1e9:.2f} G" for x in out["variants"][-3:]))
    if not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle_py as O

        nc = args.curved_cpu_cells
        mesh, pre = W.curved_cube(nc, 3, "full")
        dt = D.cfl_dt(pre, C0)
        threads = os.cpu_count() or 1
        orc = O.Oracle(mesh.raw(), dt, C0, RHO0, bcs=mesh.bcs(), upwind=(FLUX == "upwind"), num_threads=threads)
        orc.set_state(pre.initial_state([(0, 0.5, 0.5, 0.5, 2 * SIGMA ** 2, 1.0)]))
        _, sec = orc.run(0.0, 2)
        out["cpu_baseline"] = {"value": pre.ndof * 4 * 4 * 2 / sec, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"fully curved cube {nc}^3 x 6 = {pre.num_el} tets, order 3, 2 RK4 steps, "
                                         f"{sec:.1f} s"}
    return out


def parareal_section(D, args, local):
    """Learned parareal on a room with seeded box obstacles (order 3): an
    element-local MLP (3 hidden GELU layers of 256) trained on the GPU on FP64
    DG trajectories of 8 pulse positions, used as coarse propagator of
    parareal (one fine step per application) for a pulse at another
    position; fine propagator = the FP64 DG over all slices as one batch.
    Compared with parareal without the network (identity coarse propagator)
    and with the serial FP64 DG, against which the error is measured; the
    network runs with FP32 inference and with BF16 tensor-core inference."""
    from dgcuda import workloads as W

    t0 = time.time()
    cells = tuple(args.parareal_cells)
    mesh, pre, dt, ic, train = W.room(cells=cells, order=3, seed=SEED)
    nsl, sst = args.parareal_slices, args.parareal_slice_steps
    L = D.Learned(pre, C0, RHO0, flux=FLUX, width=256, hidden_layers=3, coarse_steps=1, dt=dt, seed=SEED,
                  device=local)
    for tic in train:
        L.collect(pre.initial_state([tic]), nsnap=args.parareal_train_steps, max_rows=2000)
    t_collect = time.time() - t0
    t1 = time.time()
    loss = L.train(epochs=args.parareal_epochs, batch=4096, lr=1e-3, seed=SEED)
    t_train = time.time() - t1
    u0 = pre.initial_state([ic])
    s = D.Solver(pre, C0, RHO0, flux=FLUX, device=local)
    s.set_state(u0)
    _, ms_serial = s.rk4_steps_timed(0.0, dt, nsl * sst)
    ref = s.get_state()
    s.close()
    out = {"workload": f"room 20 x 12 x 8 as {cells[0]}x{cells[1]}x{cells[2]} hexes x 6 tets minus 12 seeded box "
                       f"obstacles ({pre.num_el} tets), order 3, reflecting walls, Gaussian pulse (sigma one cell) at "
                       f"a seeded point; {nsl} slices x {sst} RK4 steps; network trained on 8 other pulse positions",
           "tets": pre.num_el, "slices": nsl, "slice_steps": sst, "tol": args.parareal_tol,
           "training": {"pairs": L.num_samples(), "epochs": args.parareal_epochs, "final_loss": loss,
                        "collect_s": t_collect, "train_s": t_train},
           "serial_fp64_ms": ms_serial}
    # one coarse application (features, network, energy-stable update) with
    # FP32 and with BF16 tensor-core inference
    napp = 200
    for mode in ("fp32", "bf16"):
        L.set_inference(mode)
        L.apply(u0, 5)
        w0 = time.perf_counter()
        L.apply(u0, napp)
        out[f"coarse_application_ms_{mode}"] = (time.perf_counter() - w0) * 1e3 / napp
    L.set_inference("fp32")
    for name, lrn, mode in (("learned", L, "fp32"), ("learned_bf16", L, "bf16"), ("identity", None, "fp32")):
        if lrn is not None:
            lrn.set_inference(mode)
        w0 = time.perf_counter()
        max_iter = nsl if args.parareal_max_iter <= 0 else min(nsl, args.parareal_max_iter)
        u, it, hist = D.parareal(pre, C0, RHO0, u0, nsl, sst, dt, tol=args.parareal_tol, max_iter=max_iter,
                                 learned=lrn, flux=FLUX)
        wall = time.perf_counter() - w0
        err = max(float(np.linalg.norm(u[q] - ref[q]) / np.linalg.norm(ref[q])) for q in range(4))
        out[name] = {"iterations": it, "wall_ms": wall * 1e3, "rel_l2_vs_serial_fp64": err,
                     "change_per_iteration": hist}
    out["coarse_step_alpha"] = L.step_stats()
    out["serial_equivalent_fine_work_dof_stages"] = pre.ndof * 4 * 4 * nsl * sst
    L.close()
    return out


def accuracy_all(D, pre, u0, dt, v0, args, local, nq):
    """Every form after the configuration's steps, relative L2 per field
    against the FP64 form (which the parity tests tie to the CPU oracle),
    computed by the library's FP64 error monitor on the device."""
    res = {}
    ref = D.Solver(pre, C0, RHO0, v0, precision="fp64", flux=FLUX, device=local)
    ref.set_state(u0)
    ref.rk4_steps(0.0, dt, args.accuracy_steps)
    res["fp64_energy_final"] = ref.monitors()[0]
    for f2 in ("mixed", "tf32x3", "fp32"):
        s = D.Solver(pre, C0, RHO0, v0, precision=f2, flux=FLUX, device=local)
        s.set_state(u0)
        s.rk4_steps(0.0, dt, args.accuracy_steps)
        rel, bad = s.error_vs(ref)
        per = [float(x) for x in rel[:nq]]
        res[f2] = {"rel_l2_vs_fp64": max(per), "per_field": per, "nonfinite": bad,
                   "meets_1e-5": bool(bad == 0 and max(per) <= 1e-5)}
        s.close()
    ref.close()
    res["steps"] = args.accuracy_steps
    res["rel_l2_vs_fp64"] = res[args.form]["rel_l2_vs_fp64"] if args.form != "fp64" else 0.0
    res["fp64_vs_oracle"] = "FP64 GPU form matches the CPU oracle to <=1e-10 relative L2 (tests/test_gpu_parity.py)"
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--accuracy-steps", type=int, default=2000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--reference-seconds", type=float, default=120.0,
                    help="time budget of the --impl reference run (sizes its per-step sample)")
    ap.add_argument("--reference-full", action="store_true",
                    help="reference arm on the full 384,000-tet workload instead of a per-step sample")
    ap.add_argument("--cells", type=int, default=NCELL, help="cube cells per side (profiling cases)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--form", choices=["mixed", "tf32x3", "fp32", "fp64"], default="mixed")
    ap.add_argument("--no-batched", action="store_true", help="skip the multi-source batch section")
    ap.add_argument("--batched-cells", type=int, default=NCELL)
    ap.add_argument("--batched-sources", type=int, default=64)
    ap.add_argument("--batched-steps", type=int, default=10)
    ap.add_argument("--batched-acc-steps", type=int, default=100)
    ap.add_argument("--batched-acc-cells", type=int, default=12,
                    help="cube cells per side of the all-members accuracy case (--batched-accuracy-only)")
    ap.add_argument("--batched-acc-all-steps", type=int, default=1000)
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven multi-mesh section")
    ap.add_argument("--uneven-meshes", type=int, default=32)
    ap.add_argument("--uneven-steps", type=int, default=500)
    ap.add_argument("--no-parareal", action="store_true", help="skip the learned parareal section")
    ap.add_argument("--parareal-cells", type=int, nargs=3, default=[20, 12, 8])
    ap.add_argument("--parareal-slices", type=int, default=16)
    ap.add_argument("--parareal-slice-steps", type=int, default=50)
    ap.add_argument("--parareal-train-steps", type=int, default=100)
    ap.add_argument("--parareal-epochs", type=int, default=10)
    ap.add_argument("--parareal-tol", type=float, default=1e-5)
    ap.add_argument("--parareal-max-iter", type=int, default=0,
                    help="parareal iterations at most (0: as many as slices, which reproduces the serial DG)")
    ap.add_argument("--no-curved", action="store_true", help="skip the curved-element section")
    ap.add_argument("--curved-cells", type=int, default=24)
    ap.add_argument("--curved-steps", type=int, default=50)
    ap.add_argument("--curved-cpu-cells", type=int, default=6)
    ap.add_argument("--curved-only", action="store_true",
                    help="run the curved-element section alone (profiling case) and print it as one JSON line")
    ap.add_argument("--parareal-only", action="store_true",
                    help="run the learned parareal section alone (profiling case) and print it as one JSON line")
    ap.add_argument("--batched-accuracy-only", action="store_true",
                    help="every member of the multi-source batch after 1000 steps against FP64 (coarser cube)")
    ap.add_argument("--batched-only", action="store_true",
                    help="run the multi-source batch section alone (profiling case) and print it as one JSON line")
    ap.add_argument("--uneven-only", action="store_true",
                    help="run the uneven multi-mesh section alone (profiling case) and print it as one JSON line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)  # at least three untimed warm-up steps
    world, rank, local, pg = dist_init()
    only = [(flag, key, fn) for flag, key, fn in
            ((args.curved_only, "curved", curved_section), (args.parareal_only, "learned_parareal", parareal_section),
             (args.batched_only, "batched", batched_section), (args.uneven_only, "uneven_batch", uneven_section),
             (args.batched_accuracy_only, "batched_accuracy_all_members", batched_accuracy_section))
            if flag]
    if only:
        import dgcuda as D

        ensure_built()
        if rank == 0:
            for _, key, fn in only:
                print(json.dumps({key: fn(D, args, local)}), flush=True)
    elif args.impl == "reference":
        reference_arm(args, world, rank, pg)
    else:
        ours_arm(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
