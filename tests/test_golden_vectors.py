"""Golden input/output vectors (tests/golden/oracle_vectors.*, written by
tests/golden/make_oracle_vectors.py from the CPU oracle): the oracle still
reproduces them, and the FP64 CUDA path matches them through the C ABI at the
1e-10 relative L2 bar."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import dgcuda as D

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "oracle_vectors.json").read_text())
ARRAYS = np.load(GOLDEN / "oracle_vectors.npz")


def _mesh(case):
    args = (*case["cells"], tuple(case["lo"]), tuple(case["hi"]))
    make = D.Mesh.box_tri if case["dim"] == 2 else D.Mesh.box_tet
    mesh = make(*args, order=case["order"], side_names=tuple(case["sides"]))
    return mesh, D.Precomp(mesh)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_reproduces_the_golden_vectors(case):
    import oracle_py as O

    mesh, pre = _mesh(case)
    u0, want = ARRAYS[case["name"] + "_u0"], ARRAYS[case["name"] + "_u"]
    assert pre.ndof == case["ndof"]
    assert np.abs(pre.initial_state([tuple(case["ic"])]) - u0).max() <= 1e-15
    orc = O.Oracle(mesh.raw(), case["dt"], case["c0"], case["rho0"], v0=tuple(case["v0"]), bcs=mesh.bcs(),
                   upwind=case["flux"] == "upwind", num_threads=1)
    orc.set_state(u0)
    orc.run(0.0, case["steps"])
    got = orc.get_state()
    for q in range(case["dim"] + 1):
        assert _rel(got[q], want[q]) <= 1e-13, q


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_fp64_matches_the_golden_vectors(case):
    _, pre = _mesh(case)
    u0, want = ARRAYS[case["name"] + "_u0"], ARRAYS[case["name"] + "_u"]
    sol = D.Solver(pre, case["c0"], case["rho0"], tuple(case["v0"]), precision="fp64", flux=case["flux"])
    try:
        sol.set_state(u0)
        sol.rk4_steps(0.0, case["dt"], case["steps"])
        got = sol.get_state()
    finally:
        sol.close()
    for q in range(case["dim"] + 1):
        assert _rel(got[q], want[q]) <= 1e-10, q
