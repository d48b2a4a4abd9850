"""Host side of the benchmark workloads (no GPU): seeded, reproducible, and
within the sizes they promise."""
from __future__ import annotations

import numpy as np

from dgcuda import workloads as W


def test_multi_source_workload():
    mesh, pre, dt, srcs, recs = W.multi_source(n=6, order=2, nsrc=5, nrec=4, sigma=0.05, seed=3)
    assert len(srcs) == 5 and len(recs) == 4
    xyz = pre.dof_coords()
    for m, (member, dofs, w, amp, freq, phase, dur) in enumerate(srcs):
        assert member == m and 2.0 <= freq <= 8.0
        assert len(dofs) == len(w) > 0
        assert np.all((w > 0) & (w <= 1.0))
        # weights follow the Gaussian of the distance to the source centre
        c = xyz[dofs[np.argmax(w)]]
        r2 = ((xyz[dofs] - c) ** 2).sum(axis=1)
        assert np.all(r2 < (2 * 3 * 0.05) ** 2)
    assert np.all((recs >= 0) & (recs < pre.ndof))
    again = W.multi_source(n=6, order=2, nsrc=5, nrec=4, sigma=0.05, seed=3)
    assert np.array_equal(again[4], recs) and again[2] == dt


def test_uneven_workload_sizes_and_orders():
    meshes, pres, phys, dts, srcs = W.uneven(nmesh=5, seed=11, min_tets=600, max_tets=6000, orders=(2, 3))
    assert len(pres) == 5 and len(srcs) == 5
    for p in pres:
        assert 600 <= p.num_el <= 6000 and p.order in (2, 3)
    assert np.all(dts > 0)
    again = W.uneven(nmesh=5, seed=11, min_tets=600, max_tets=6000, orders=(2, 3))
    assert [p.num_el for p in again[1]] == [p.num_el for p in pres]


def test_room_with_obstacles():
    mesh, pre, dt, ic, train = W.room(cells=(8, 6, 4), size=(8.0, 6.0, 4.0), order=1, nobst=3, seed=5, ntrain=3)
    assert pre.num_el < 8 * 6 * 4 * 6  # cells removed
    assert len(train) == 3
    # the pulse sits at a cell centre that is not an obstacle: nodes around it exist
    xyz = pre.dof_coords()
    d = np.sqrt(((xyz - np.array(ic[1:4])) ** 2).sum(axis=1)).min()
    assert d < 1.0
