"""Host logic of the GPU path without a GPU: the element-centric layout that
dg_create uploads, driven through a NumPy model of the stage kernel's
arithmetic, reproduces the oracle's right-hand side (FP64 roundoff)."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
import kernel_model as KM
import oracle_py as O

C0, RHO0 = 340.0, 1.225


@pytest.mark.parametrize("dim,order,v0,flux", [
    (2, 1, (0.0, 0.0, 0.0), "reference"), (2, 3, (30.0, -20.0, 0.0), "reference"),
    (2, 4, (0.0, 0.0, 0.0), "upwind"), (2, 5, (10.0, 0.0, 0.0), "reference"),
    (3, 1, (0.0, 0.0, 0.0), "reference"), (3, 2, (50.0, 0.0, 10.0), "reference"),
    (3, 3, (100.0, 0.0, 0.0), "reference"), (3, 3, (0.0, 0.0, 0.0), "upwind"),
    (3, 4, (0.0, 0.0, 0.0), "reference"), (3, 5, (20.0, 0.0, 0.0), "upwind")])
def test_layout_model_matches_oracle_rhs(dim, order, v0, flux):
    if dim == 2:
        m = D.Mesh.box_tri(3, 2, order=order, side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    else:
        m = D.Mesh.box_tet(2, 2, 1, order=order, side_names=("Absorbing", "Reflecting") * 3)
    pre = D.Precomp(m)
    lay = pre.layout(flux)
    orc = O.Oracle(m.raw(), 1e-4, C0, RHO0, v0=v0, bcs=m.bcs(), upwind=(flux == "upwind"))
    u = np.random.default_rng(order).standard_normal((4, pre.ndof))
    if dim == 2:
        u[3] = 0
    ro = orc.rhs(u)
    rm = KM.rhs(lay, u, 1e-4, C0, RHO0, v0)
    tol = 1e-12 if order <= 4 else 1e-11
    for q in range(dim + 1):
        assert np.linalg.norm(rm[q] - ro[q]) <= tol * np.linalg.norm(ro[q])
    if dim == 2:
        assert np.all(ro[3] == 0)


def test_layout_connectivity_words():
    m = D.Mesh.box_tet(2, 1, 1, order=3, side_names=("Absorbing", "Reflecting") * 3)
    pre = D.Precomp(m)
    lay = pre.layout("reference")
    conn = lay["conn"]
    kind = (conn[..., 1] >> 5) & 3
    nb = conn[..., 0]
    assert np.all((kind == 0) == (nb >= 0))
    arr = pre.arrays()
    nbnd = int(arr["f_is_boundary"].sum())
    assert int((kind > 0).sum()) == nbnd
    # reference sign for 3D order 3: fc = -1, first-point normal outward of
    # the first neighbour -> negative jump sign on every interior face
    assert np.all((conn[..., 1][kind == 0] & 128) != 0)
    up = pre.layout("upwind")["conn"]
    assert np.all((up[..., 1][kind == 0] & 128) == 0)
    # outward unit normals, positive area ratios
    n = lay["fgeo"][..., :3]
    assert np.allclose(np.linalg.norm(n, axis=-1), 1.0)
    assert np.all(lay["fgeo"][..., 3] > 0)
