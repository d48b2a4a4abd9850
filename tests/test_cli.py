"""The drop-in command line: dgalerkin mesh.msh config.conf writes the
reference's Pressure / Density / Velocity ElementNodeData views at timeRate;
a saved frame matches the oracle after the same number of steps."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O

pytestmark = pytest.mark.gpu

CONF = """timeStart=0
timeEnd={tend}
timeStep={dt}
timeRate={rate}
elementType=Lagrange
timeIntMethod={method}
Reflecting = Reflecting
Absorbing = Absorbing
numThreads=1
v0_x = 0
v0_y = 0
v0_z = 0
rho0 = 1.225
c0 = 340
initialCondtition1 = gaussian, 0.1,-0.1,0,0.05,1
source1 = monopole, -0.3,0.2,0, 0.2, 1,900,0,{sdur}
saveFile={save}
"""


def read_views(path):
    text = open(path).read().split("$ElementNodeData\n")[1:]
    views = {}
    for blk in text:
        lines = blk.split("\n")
        name = lines[1].strip('"')
        t = float(lines[3])
        step = int(lines[5])
        ncomp = int(lines[6])
        nel = int(lines[7])
        vals = [list(map(float, lines[8 + e].split()[2:])) for e in range(nel)]
        views.setdefault(name, []).append((step, t, ncomp, np.array(vals)))
    return views


def test_cli_matches_oracle(tmp_path):
    mesh = D.Mesh.box_tri(4, 4, (-1, -1), (1, 1), order=2,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    msh = tmp_path / "box.msh"
    mesh.write_msh(msh)
    m2 = D.Mesh.read_msh(msh)
    pre = D.Precomp(m2)
    dt = D.cfl_dt(pre, 340.0)
    conf = tmp_path / "c.conf"
    save = tmp_path / "out.msh"
    conf.write_text(CONF.format(tend=(30 - 0.5) * dt, dt=repr(dt), rate=repr(10 * dt * 0.999), sdur=repr(12 * dt),
                                save=save, method="Runge-Kutta"))
    exe = D.PKG / "lib" / "dgalerkin"
    r = subprocess.run([str(exe), str(msh), str(conf)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    views = read_views(save)
    assert set(views) == {"Pressure", "Density", "Velocity"}
    steps = [s for s, _, _, _ in views["Pressure"]]
    assert steps[0] == 0 and len(steps) >= 3
    step, t, ncomp, p = views["Pressure"][2]
    # the same run on the oracle
    cfg = D.Config.parse(conf, m2)
    orc = O.Oracle(m2.raw(), dt, 340.0, 1.225, bcs=cfg.bcs, sources=cfg.sources)
    orc.set_state(pre.initial_state(cfg.ics))
    orc.run(0.0, step)
    ref = orc.get_state()[0].reshape(pre.num_el, pre.np)
    assert np.linalg.norm(p - ref) <= 1e-10 * np.linalg.norm(ref)
    rho = views["Density"][2][3]
    assert np.allclose(rho, p / 340.0 ** 2, rtol=1e-15)
    vel = views["Velocity"][2][3].reshape(pre.num_el, pre.np, 3)
    assert np.all(vel[..., 2] == 0)


def test_cli_curved_mesh_matches_oracle(tmp_path):
    """A curved order-3 .msh (nodes moved by a smooth map): the executable
    runs it with per-point geometry and a saved frame matches the oracle."""
    mesh = D.Mesh.box_tri(4, 4, (-1, -1), (1, 1), order=3,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    mesh.warp(lambda x: np.stack([x[:, 0] + 0.05 * np.sin(np.pi * x[:, 1]),
                                  x[:, 1] + 0.05 * np.sin(np.pi * x[:, 0]), x[:, 2]], 1))
    msh = tmp_path / "curved.msh"
    mesh.write_msh(msh)
    m2 = D.Mesh.read_msh(msh)
    pre = D.Precomp(m2)
    assert pre.num_curved == pre.num_el
    dt = D.cfl_dt(pre, 340.0)
    conf = tmp_path / "c.conf"
    save = tmp_path / "out.msh"
    conf.write_text(CONF.format(tend=(30 - 0.5) * dt, dt=repr(dt), rate=repr(10 * dt * 0.999), sdur=repr(8 * dt),
                                save=save, method="Runge-Kutta"))
    exe = D.PKG / "lib" / "dgalerkin"
    r = subprocess.run([str(exe), str(msh), str(conf)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    step, t, ncomp, p = read_views(save)["Pressure"][2]
    cfg = D.Config.parse(conf, m2)
    orc = O.Oracle(m2.raw(), dt, 340.0, 1.225, bcs=cfg.bcs, sources=cfg.sources)
    orc.set_state(pre.initial_state(cfg.ics))
    orc.run(0.0, step)
    ref = orc.get_state()[0].reshape(pre.num_el, pre.np)
    assert np.linalg.norm(p - ref) <= 1e-10 * np.linalg.norm(ref)


def test_cli_forward_euler_and_unknown_method(tmp_path):
    """timeIntMethod = Euler1 runs forward Euler (dgalerkin.cpp:55-56); a name
    the reference does not know runs nothing and writes no views."""
    mesh = D.Mesh.box_tri(4, 4, (-1, -1), (1, 1), order=3,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    msh = tmp_path / "box.msh"
    mesh.write_msh(msh)
    m2 = D.Mesh.read_msh(msh)
    pre = D.Precomp(m2)
    dt = 0.2 * D.cfl_dt(pre, 340.0)
    exe = D.PKG / "lib" / "dgalerkin"
    conf = tmp_path / "e.conf"
    save = tmp_path / "euler.msh"
    conf.write_text(CONF.format(tend=(20 - 0.5) * dt, dt=repr(dt), rate=repr(7 * dt * 0.999), sdur=repr(5 * dt),
                                save=save, method="Euler1"))
    r = subprocess.run([str(exe), str(msh), str(conf)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    step, t, ncomp, p = read_views(save)["Pressure"][2]
    cfg = D.Config.parse(conf, m2)
    orc = O.Oracle(m2.raw(), dt, 340.0, 1.225, bcs=cfg.bcs, sources=cfg.sources)
    orc.set_method("Euler1")
    orc.set_state(pre.initial_state(cfg.ics))
    orc.run(0.0, step)
    ref = orc.get_state()[0].reshape(pre.num_el, pre.np)
    assert np.linalg.norm(p - ref) <= 1e-10 * np.linalg.norm(ref)

    conf2 = tmp_path / "u.conf"
    save2 = tmp_path / "none.msh"
    conf2.write_text(CONF.format(tend=5 * dt, dt=repr(dt), rate=repr(dt), sdur="0", save=save2,
                                 method="Leapfrog"))
    r = subprocess.run([str(exe), str(msh), str(conf2)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert not save2.exists()
