"""Writes tests/golden/reference_meshes.json: element, face and boundary-face
counts of the reference's shipped gmsh meshes (doc/2d, doc/3d), read with this
project's MSH 4.0 reader.  The count of holes comes from the Euler
characteristic of the 2D meshes.  Give it the reference checkout:
    python tests/golden/make_reference_mesh_counts.py /path/to/reference
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "dgfem-acoustic_gb300"))
import dgcuda as D  # noqa: E402

if len(sys.argv) != 2:
    sys.exit("usage: make_reference_mesh_counts.py /path/to/reference")
ref = Path(sys.argv[1])
out = {}
for n in ["doc/2d/square.msh", "doc/2d/disk.msh", "doc/2d/square_reflection.msh", "doc/2d/room.msh",
          "doc/3d/cube.msh", "doc/3d/sphere.msh"]:
    m = D.Mesh.read_msh(ref / n)
    r = m.raw()
    bcs = [(int(t), nm.startswith("Reflecting")) for d, t, nm in zip(r["phys_dim"], r["phys_tag"], r["phys_name"])
           if d == r["dim"] - 1]
    pre = D.Precomp(m, bcs)
    a = pre.arrays()
    rec = {"dim": r["dim"], "order": r["order"], "num_el": pre.num_el, "f_num": pre.f_num,
           "boundary_faces": int(a["f_is_boundary"].sum()), "phys": sorted(set(r["phys_name"]))}
    if r["dim"] == 2:
        V = len(np.unique(r["el_nodes"][:, :3]))
        chi = V - pre.f_num + pre.num_el
        if chi != 1:
            rec["holes"] = 1 - chi
    out[Path(n).name] = rec
    print(Path(n).name, rec)
(Path(__file__).parent / "reference_meshes.json").write_text(json.dumps(out, indent=1) + "\n")
