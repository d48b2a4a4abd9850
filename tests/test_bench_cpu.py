"""bench.py on the CPU: the rank aggregation of the replica path (gloo,
world size 2) and the reference arm (the oracle on the host cores) launched
by torchrun with two ranks, where rank 0 alone prints the JSON line."""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out) -> None:
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, local, pg = bench.dist_init()
    try:
        bench.barrier(pg)
        # each rank's timed milliseconds and processed units, as in the replica path
        ms_max = bench.allreduce_max(pg, 10.0 + rank)
        units = bench.allreduce_sum(pg, 1000.0 * (rank + 1))
        bench.barrier(pg)
        out.put((r, w, local, ms_max, units))
    finally:
        pg.destroy_process_group()


def test_replica_aggregation_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], codes
    res = sorted(q.get(timeout=5) for _ in range(2))
    # every rank sees the slowest rank's time and the units of all ranks
    assert [x[:3] for x in res] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, ms_max, units in res:
        assert ms_max == 11.0
        assert units == 3000.0


def test_reference_arm_under_torchrun_prints_one_line_from_rank0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--reference-seconds", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["n_gpus"] == 2 and d["steps"] == 1 and d["warmup"] == 3
    assert d["unit"] == "DOF-stage/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    for key in ("metric", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in d
    assert d["config"]["tets"] == 384000 and d["config"]["fields"] == 4
    assert d["sample"] and d["sample_reason"]


def test_reference_arm_inputs_match_the_product_workload():
    """The reference arm builds its mesh, initial state and time step without
    the product library (oracle_box / oracle_workload).  On a small case they
    equal the product's box generator and precompute: same element node
    coordinates in the same order, same initial state, same time step, and
    the oracle's right-hand side is the same on either mesh."""
    sys.path.insert(0, str(ROOT))
    import numpy as np

    import bench
    import dgcuda as D
    import oracle_py as O

    n = 3
    raw, u0, dt, v0 = bench.oracle_workload(n)
    mesh, pre, v0p, dtp, ic = bench.workload(n)
    X = raw["xyz"][raw["el_nodes"] - 1].reshape(-1, 3)
    assert np.abs(X - pre.dof_coords()).max() <= 1e-15
    assert abs(dt - dtp) <= 1e-14 * dtp and tuple(v0) == tuple(v0p)
    up = pre.initial_state([ic])
    assert np.abs(u0 - up).max() <= 1e-15
    a = O.Oracle(raw, dt, 340.0, 1.225, v0=v0, upwind=True)
    b = O.Oracle(mesh.raw(), dt, 340.0, 1.225, v0=v0, bcs=mesh.bcs(), upwind=True)
    u = np.random.default_rng(1).standard_normal((4, pre.ndof))
    ra, rb = a.rhs(u), b.rhs(u)
    assert np.abs(ra - rb).max() <= 1e-12 * np.abs(rb).max()
    # congruent cells: the time step scales with the cell size, which is how
    # the reference arm states the full workload's dt from its sample
    _, _, dt8 = bench.oracle_box(8)
    assert abs(dt * n / 8 - dt8) <= 1e-15 * dt8
