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
