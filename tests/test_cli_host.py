"""The dgalerkin command line up to the point where it needs a GPU: argument
count (E2BIG, as dgalerkin.cpp:11-12), unreadable inputs, and a run whose
timeIntMethod the reference does not know (dgalerkin.cpp:55-58: the mesh and
configuration are read and the Mesh precompute runs, then nothing is solved
and no views are written), which exercises the whole host side, binary
.msh input included, without a device."""
from __future__ import annotations

import errno
import subprocess

import pytest

import dgcuda as D

EXE = D.PKG / "lib" / "dgalerkin"

CONF = """timeStart=0
timeEnd=0.001
timeStep=0.0001
timeRate=0.0005
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
saveFile={save}
"""


def run(*args):
    return subprocess.run([str(EXE), *map(str, args)], capture_output=True, text=True, timeout=120)


def test_argument_count():
    for args in ((), ("only-one",), ("a", "b", "c")):
        assert run(*args).returncode == errno.E2BIG


def test_unreadable_inputs(tmp_path):
    conf = tmp_path / "c.conf"
    conf.write_text(CONF.format(method="Runge-Kutta", save=tmp_path / "out.msh"))
    r = run(tmp_path / "missing.msh", conf)
    assert r.returncode != 0 and "Error" in r.stderr
    mesh = D.Mesh.box_tri(2, 2, order=2)
    msh = tmp_path / "m.msh"
    mesh.write_msh(msh)
    r = run(msh, tmp_path / "missing.conf")
    assert r.returncode != 0 and "Error" in r.stderr


@pytest.mark.parametrize("binary", [False, True])
def test_unknown_method_runs_the_host_side_only(tmp_path, binary):
    from msh_binary import parse_msh41, write_msh41_binary

    mesh = D.Mesh.box_tet(2, 2, 2, order=2, side_names=("Reflecting", "Absorbing") * 3)
    msh = tmp_path / "ascii.msh"
    mesh.write_msh(msh)
    if binary:
        b = tmp_path / "binary.msh"
        write_msh41_binary(parse_msh41(msh), b)
        msh = b
    save = tmp_path / "views.msh"
    save.write_text("stale")  # the reference removes saveFile before it starts
    conf = tmp_path / "c.conf"
    conf.write_text(CONF.format(method="Leapfrog", save=save))
    r = run(msh, conf)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Number of Elements : 48" in r.stdout
    assert "Element Order : 2" in r.stdout
    assert "nothing to run" in r.stdout
    assert not save.exists()
