"""Benchmark of the DG acoustic RK4 right-hand side on one GB300.

Workload (the configuration the metric is quoted on): unit cube as a 40^3 hex
grid, each hex split into 6 tetrahedra (384,000 tets), order 3 (Np = 20),
linearised Euler with uniform mean flow Mach 0.3 along x (c0 = 340,
rho0 = 1.225), absorbing boundaries, Gaussian pressure pulse sigma = 0.05 at
a seeded interior point, dt from CFL 0.5.  Four evolved fields (p, vx, vy,
vz); density is p/c0^2 at output.  A step is one classical RK4 time step
(four fused stage launches).  The chosen form is FP32 state and flux with
FP64 geometry factors; the plain FP64 form is measured beside it, and the
chosen form's error against FP64 is measured after the configuration's 2000
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
def stage_bytes(pre, real_bytes: int) -> list[float]:
    """Algorithmic HBM bytes of each fused stage launch (unique bytes: state
    reads/writes, geometry once; neighbour traces are L2 re-reads).
    Stage 1 reads u, writes acc and w; stages 2-3 read w, u, acc and write
    acc, w; stage 4 reads w, u, acc and writes u."""
    nq = pre.dim + 1
    n = pre.ndof * nq
    geo = pre.num_el * (pre.dim * pre.dim * 8 + pre.nf * 4 * real_bytes + pre.nf * 8)
    return [n * real_bytes * k + geo for k in (3, 5, 5, 4)]


# ------------------------------------------------------------------ CPU (oracle)
def oracle_sample_rate(n: int, steps: int, threads: int, dedup: bool = False):
    """Faithful CPU restatement timed on an n^3 x 6 sample of the workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O

    mesh, pre, v0, dt, ic = workload(n)
    orc = O.Oracle(mesh.raw(), dt, C0, RHO0, v0=v0, bcs=mesh.bcs(), upwind=(FLUX == "upwind"),
                   num_threads=threads)
    orc.set_state(pre.initial_state([ic]))
    _, sec = orc.run(0.0, steps, dedup=dedup)
    dofstage = pre.ndof * 4 * 4 * steps
    return dofstage / sec, sec, pre


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
    rate, sec, pre = oracle_sample_rate(n, steps, threads)
    rate_dedup, _, _ = oracle_sample_rate(n, max(1, steps // 2), threads, dedup=True)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n}^3 x 6 = {pre.num_el} tets of the same workload (order 3, Mach 0.3, absorbing), "
                      f"{steps} RK4 steps, {sec:.1f} s, faithful nested-OpenMP face loop",
            "dedup_face_loop_value": rate_dedup}


def reference_arm(args, world, rank, pg):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    total = args.steps + args.warmup
    # per-step sample sized so the whole run stays within about two minutes
    _, sec4, _ = oracle_sample_rate(4, 1, threads)
    n = 2
    for cand in (3, 4, 6, 8, 10, 12, 16):
        if sec4 * (cand / 4) ** 3 * total <= 120.0:
            n = cand
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O

    mesh, pre, v0, dt, ic = workload(n)
    orc = O.Oracle(mesh.raw(), dt, C0, RHO0, v0=v0, bcs=mesh.bcs(), upwind=(FLUX == "upwind"), num_threads=threads)
    orc.set_state(pre.initial_state([ic]))
    t = 0.0
    if args.warmup:
        t, _ = orc.run(t, args.warmup)
    t, sec = orc.run(t, args.steps)
    dofstage = pre.ndof * 4 * 4 * args.steps
    value = dofstage / sec
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "reference CPU algorithm (faithful C++/OpenMP restatement)",
                       "sample": f"{n}^3 x 6 = {pre.num_el} tets per step", "flux_sign": FLUX},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n}^3 x 6 = {pre.num_el} tets, {args.steps} timed RK4 steps, {sec:.1f} s"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
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

    sol = D.Solver(pre, C0, RHO0, v0, precision="fp32", flux=FLUX, device=local)
    sol.set_state(u0)
    t = 0.0
    if args.warmup:
        t = sol.rk4_steps(t, dt, args.warmup)

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

    # per-kernel timing of the same workload (events around every launch)
    _, prof = sol.profile_steps(t, dt, min(args.steps, 200))
    real = 4
    sb = stage_bytes(pre, real)
    avg_ms = [prof["stage_ms"][s] / max(prof["stage_launches"][s], 1) for s in range(4)]
    achieved = sum(sb) / (sum(avg_ms) * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic("stage_kernel_cube40_p3_fp32.md")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": sum(sb) / 4, "stage_ms": avg_ms,
                "kernel": "stage_kernel<3,3,float> (fused volume + face flux + lift + RK4 update)"}

    # end to end: every step set_state from pinned host memory, one step,
    # get_state into pinned host memory, through the C ABI
    n_e2e = 0 if args.no_e2e else args.steps
    L = D.lib()
    nbytes = 4 * pre.ndof * 8
    hin = L.dg_host_alloc(nbytes)
    hout = L.dg_host_alloc(nbytes)
    if not hin or not hout:
        raise RuntimeError("pinned host allocation failed")
    import ctypes as C

    uin = np.ctypeslib.as_array((C.c_double * (4 * pre.ndof)).from_address(hin)).reshape(4, pre.ndof)
    uout = np.ctypeslib.as_array((C.c_double * (4 * pre.ndof)).from_address(hout)).reshape(4, pre.ndof)
    uin[:] = u0
    barrier(pg)
    sol.synchronize()
    w0 = time.perf_counter()
    te = 0.0
    for _ in range(n_e2e):
        sol.set_state(uin)
        te = sol.rk4_steps(te, dt, 1)
        sol.get_state(uout)
    sol.synchronize()
    w1 = time.perf_counter()
    barrier(pg)
    e2e_s = allreduce_max(pg, w1 - w0)
    e2e_value = allreduce_sum(pg, dof_stage_per_step * n_e2e) / e2e_s if n_e2e else None
    L.dg_host_free(hin)
    L.dg_host_free(hout)

    # plain FP64 form on the same workload
    plain_info, acc = None, None
    if args.no_plain:
        args.accuracy_steps = 0
    plain = None if args.no_plain else D.Solver(pre, C0, RHO0, v0, precision="fp64", flux=FLUX, device=local)
    if plain is not None:
        plain_info = plain_form(plain, u0, dt, args, dof_stage_per_step)
    if plain is not None and args.accuracy_steps > 0:
        acc = accuracy(D, pre, plain, u0, dt, v0, args, local, nq)
    if plain is not None:
        plain.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.cpu_seconds)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if args.cells == NCELL else WORKLOAD + f" (profiling case: {args.cells}^3 cells)",
                   "form": "FP32 state and flux, FP64 geometry factors, fused stage kernel",
                   "tets": pre.num_el, "dofs_per_field": pre.ndof, "fields": nq, "dt": dt, "flux_sign": FLUX,
                   "l2": "inputs larger than L2 (FP32 state 4 x %.0f MB)" % (pre.ndof * nq * 4 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "plain_fp64": plain_info,
        "accuracy": acc,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": n_e2e, "how": "per step: dg_set_state from pinned host, dg_rk4_steps(1), dg_get_state"},
        "clocks": clk.summary(),
        "gpu_launches": 4 * args.steps,
        "monitors": {"energy": e, "nonfinite": bad},
    }
    if plain_info:
        plain_info["chosen_over_plain"] = value / plain_info["value"]
    print(json.dumps(line), flush=True)


def plain_form(plain, u0, dt, args, dof_stage_per_step):
    plain.set_state(u0)
    tp = plain.rk4_steps(0.0, dt, 3)
    n_plain = max(5, min(args.steps, 40))
    tp, pms = plain.rk4_steps_timed(tp, dt, n_plain)
    _, pprof = plain.profile_steps(tp, dt, 5)
    pavg = [pprof["stage_ms"][s] / max(pprof["stage_launches"][s], 1) for s in range(4)]
    return {"value": dof_stage_per_step * n_plain / (pms * 1e-3), "unit": UNIT, "ms_per_step": pms / n_plain,
            "stage_ms": pavg}


def accuracy(D, pre, plain, u0, dt, v0, args, local, nq):
    a32 = D.Solver(pre, C0, RHO0, v0, precision="fp32", flux=FLUX, device=local)
    a32.set_state(u0)
    plain.set_state(u0)
    a32.rk4_steps(0.0, dt, args.accuracy_steps)
    plain.rk4_steps(0.0, dt, args.accuracy_steps)
    r32, r64 = a32.get_state(), plain.get_state()
    per = [float(np.linalg.norm(r32[q] - r64[q]) / np.linalg.norm(r64[q])) for q in range(nq)]
    e64, _, _ = plain.monitors()
    a32.close()
    return {"rel_l2_vs_fp64": max(per), "per_field": per, "steps": args.accuracy_steps, "fp64_energy_final": e64,
            "fp64_vs_oracle": "FP64 GPU form matches the CPU oracle to <=1e-10 relative L2 "
                              "(tests/test_gpu_parity.py)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--accuracy-steps", type=int, default=2000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cells", type=int, default=NCELL, help="cube cells per side (profiling cases)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)  # at least three untimed warm-up steps
    world, rank, local, pg = dist_init()
    if args.impl == "reference":
        reference_arm(args, world, rank, pg)
    else:
        ours_arm(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
