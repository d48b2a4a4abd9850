"""Writes tests/golden/oracle_vectors.{json,npz}: small seeded cases run
through the CPU oracle (the restatement of the reference's solver), stored
as golden input/output vectors.  The cases are described in the JSON (mesh
generator arguments, medium, mean flow, flux mode, initial condition, dt,
steps); the NPZ holds each case's initial state and its state after the
steps, [4][ndof] in the reference layout.

    python tests/golden/make_oracle_vectors.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "dgfem-acoustic_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

CASES = [
    {"name": "tri_p3_meanflow_reference_sign", "dim": 2, "cells": [4, 4], "lo": [-1.0, -1.0], "hi": [1.0, 1.0],
     "order": 3, "sides": ["Reflecting", "Absorbing", "Reflecting", "Absorbing"], "c0": 340.0, "rho0": 1.225,
     "v0": [60.0, -30.0, 0.0], "flux": "reference", "ic": [0, 0.1, -0.1, 0.0, 0.05, 1.0], "cfl_fraction": 1.0,
     "steps": 20},
    {"name": "tet_p2_meanflow_upwind", "dim": 3, "cells": [2, 2, 2], "lo": [0.0, 0.0, 0.0], "hi": [1.0, 1.0, 1.0],
     "order": 2, "sides": ["Reflecting", "Absorbing"] * 3, "c0": 340.0, "rho0": 1.225, "v0": [102.0, 0.0, 0.0],
     "flux": "upwind", "ic": [0, 0.4, 0.5, 0.6, 0.02, 1.0], "cfl_fraction": 0.5, "steps": 20},
]


def build_case(D, case):
    if case["dim"] == 2:
        mesh = D.Mesh.box_tri(*case["cells"], tuple(case["lo"]), tuple(case["hi"]), order=case["order"],
                              side_names=tuple(case["sides"]))
    else:
        mesh = D.Mesh.box_tet(*case["cells"], tuple(case["lo"]), tuple(case["hi"]), order=case["order"],
                              side_names=tuple(case["sides"]))
    return mesh, D.Precomp(mesh)


def main() -> None:
    import dgcuda as D
    import oracle_py as O

    out, arrays = [], {}
    for case in CASES:
        mesh, pre = build_case(D, case)
        dt = case["cfl_fraction"] * D.cfl_dt(pre, case["c0"])
        u0 = pre.initial_state([tuple(case["ic"])])
        orc = O.Oracle(mesh.raw(), dt, case["c0"], case["rho0"], v0=tuple(case["v0"]), bcs=mesh.bcs(),
                       upwind=case["flux"] == "upwind", num_threads=1)
        orc.set_state(u0)
        orc.run(0.0, case["steps"])
        arrays[case["name"] + "_u0"] = u0
        arrays[case["name"] + "_u"] = orc.get_state()
        out.append(dict(case, dt=dt, ndof=pre.ndof))
    (HERE / "oracle_vectors.json").write_text(json.dumps(out, indent=1) + "\n")
    np.savez_compressed(HERE / "oracle_vectors.npz", **arrays)


if __name__ == "__main__":
    main()
