"""Seeded synthetic workloads of the batched forms.

multi_source: one mesh, many Gaussian-in-space hard sources (one per batch
member) with sine time signals, and pressure receivers.
uneven: many box meshes of seeded sizes and orders, one Gaussian source
each, reflecting and absorbing sides mixed.
curved_cube: a unit cube whose nodes are moved by a smooth map, so that all
or half of its (isoparametric) elements are curved.
"""
from __future__ import annotations

import numpy as np

from . import Mesh, Precomp, cfl_dt

C0, RHO0 = 340.0, 1.225


def multi_source(n: int = 40, order: int = 4, nsrc: int = 64, nrec: int = 16, sigma: float = 0.03,
                 seed: int = 2026, side_names=("Absorbing",) * 6):
    """Unit cube of n^3 hexes x 6 tets; nsrc sources at positions uniform in
    [0.1, 0.9]^3, each a Gaussian of width sigma in space (nodes within
    3 sigma) times sin(2 pi f t), f uniform in [2, 8]; nrec receivers at the
    nodes nearest to seeded points.  Returns (mesh, pre, dt, sources,
    receivers) with sources as (member, dofs, weights, amp, freq, phase,
    duration) tuples."""
    mesh = Mesh.box_tet(n, n, n, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), order=order, side_names=side_names)
    pre = Precomp(mesh)
    dt = cfl_dt(pre, C0)
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.1, 0.9, (nsrc, 3))
    freq = rng.uniform(2.0, 8.0, nsrc)
    srcs = []
    for m in range(nsrc):
        dofs, w = pre.gaussian_source(*pos[m], sigma)
        srcs.append((m, dofs, w, 1.0, float(freq[m]), 0.0, 1e30))
    xyz = pre.dof_coords()
    rec_pts = rng.uniform(0.1, 0.9, (nrec, 3))
    recs = np.array([int(np.argmin(((xyz - p) ** 2).sum(axis=1))) for p in rec_pts], dtype=np.int32)
    return mesh, pre, dt, srcs, recs


def uneven(nmesh: int = 32, seed: int = 2026, h: float = 0.025, min_tets: int = 5000, max_tets: int = 300000,
           orders=(2, 3, 4, 5)):
    """nmesh boxes with side lengths uniform in [0.5, 3] (seeded), split into
    hexes of size h (coarsened where needed so that every mesh holds between
    min_tets and max_tets tets, target log-uniform in that range) x 6 tets;
    order uniform in `orders`; each side reflecting or absorbing at random; one
    Gaussian source (sigma = 2 cells) per mesh.  Returns (meshes, pres, phys,
    dts, sources) with sources as (mesh, dofs, weights, amp, freq, phase,
    duration)."""
    rng = np.random.default_rng(seed)
    meshes, pres, phys, dts, srcs = [], [], [], [], []
    for i in range(nmesh):
        L = rng.uniform(0.5, 3.0, 3)
        target = float(np.exp(rng.uniform(np.log(min_tets), np.log(max_tets))))
        hh = max(h, (6.0 * L.prod() / target) ** (1.0 / 3.0))
        cells = [max(1, int(round(x / hh))) for x in L]
        while 6 * cells[0] * cells[1] * cells[2] > max_tets:
            k = int(np.argmax(cells))
            cells[k] -= 1
        while 6 * cells[0] * cells[1] * cells[2] < min_tets:
            k = int(np.argmin(cells))
            cells[k] += 1
        order = int(rng.choice(orders))
        names = tuple("Reflecting" if rng.uniform() < 0.5 else "Absorbing" for _ in range(6))
        mesh = Mesh.box_tet(*cells, (0.0, 0.0, 0.0), tuple(L), order=order, side_names=names)
        pre = Precomp(mesh)
        meshes.append(mesh)
        pres.append(pre)
        phys.append((C0, RHO0, (0.0, 0.0, 0.0)))
        dts.append(cfl_dt(pre, C0))
        pos = rng.uniform(0.2, 0.8, 3) * L
        sigma = 2.0 * float(L.max() / max(cells))
        dofs, w = pre.gaussian_source(*pos, sigma)
        srcs.append((i, dofs, w, 1.0, float(rng.uniform(2.0, 8.0)), 0.0, 1e30))
    return meshes, pres, phys, np.array(dts), srcs


def room(cells=(20, 12, 8), size=(20.0, 12.0, 8.0), order: int = 3, nobst: int = 12, seed: int = 2026,
         ntrain: int = 8):
    """Room of the given size as a hex grid split into tets, with nobst seeded
    box obstacles (1-3 cells per side, cells removed, reflecting), reflecting
    walls.  Returns (mesh, pre, dt, ic, train_ics): ic is a Gaussian pressure
    pulse (sigma = one cell) at a seeded free point, train_ics ntrain more."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = cells
    h = np.array(size) / np.array(cells)
    gone = np.zeros(cells[::-1], dtype=bool)  # [k][j][i]
    for _ in range(nobst):
        ext = rng.integers(1, 4, 3)
        at = [int(rng.integers(0, c - e + 1)) for c, e in zip(cells, ext)]
        gone[at[2]:at[2] + ext[2], at[1]:at[1] + ext[1], at[0]:at[0] + ext[0]] = True
    removed = [int(i + nx * (j + ny * k)) for k, j, i in zip(*np.nonzero(gone))]
    mesh = Mesh.box_tet(nx, ny, nz, (0.0, 0.0, 0.0), tuple(size), order=order, side_names=("Reflecting",) * 6,
                        removed=removed, obstacle_name="Reflecting")
    pre = Precomp(mesh)
    dt = cfl_dt(pre, C0)
    sigma = float(h.max())

    def free_point():
        while True:
            c = rng.integers(1, np.array(cells) - 1)
            if not gone[c[2], c[1], c[0]]:
                return tuple((c + 0.5) * h)

    ic = (0, *free_point(), 2 * sigma ** 2, 1.0)
    train = [(0, *free_point(), 2 * sigma ** 2, 1.0) for _ in range(ntrain)]
    return mesh, pre, dt, ic, train


def curved_cube(n: int = 24, order: int = 3, kind: str = "full", amplitude: float = 0.02,
                side_names=("Absorbing",) * 6):
    """Unit cube of n^3 hexes x 6 tets, nodes moved by a smooth map.  kind
    "full": x += a sin(pi y) sin(pi z), y += a sin(pi x) cos(pi z),
    z += a sin(2x + y), which curves every element; "half": y and z move by
    a (x - 1/2)^3 sin / cos terms for x > 1/2 only, so the elements with
    x <= 1/2 stay straight; "none": the straight cube.  Returns (mesh, pre)."""
    mesh = Mesh.box_tet(n, n, n, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), order=order, side_names=side_names)
    a = amplitude
    if kind == "full":
        def fn(x):
            y = x.copy()
            y[:, 0] = x[:, 0] + a * np.sin(np.pi * x[:, 1]) * np.sin(np.pi * x[:, 2])
            y[:, 1] = x[:, 1] + a * np.sin(np.pi * x[:, 0]) * np.cos(np.pi * x[:, 2])
            y[:, 2] = x[:, 2] + a * np.sin(2 * x[:, 0] + x[:, 1])
            return y
        mesh.warp(fn)
    elif kind == "half":
        def fn(x):
            y = x.copy()
            s = np.clip(x[:, 0] - 0.5, 0.0, None) ** 3
            y[:, 1] = x[:, 1] + 8 * a * s * np.sin(np.pi * x[:, 2])
            y[:, 2] = x[:, 2] + 8 * a * s * np.cos(np.pi * x[:, 1])
            return y
        mesh.warp(fn)
    elif kind != "none":
        raise ValueError("kind must be full, half or none")
    return mesh, Precomp(mesh)
