"""The .conf parser keeps the reference's keys and quirks
(configParser.cpp:30-150)."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D

CONF = """[Config]
# comment
timeStart=0
timeEnd = 0.2
timeStep=1e-5
timeRate=0.0001
elementType=Lagrange
timeIntMethod=Runge-Kutta
Reflecting = Reflecting
Absorbing = Absorbing
numThreads=1
v0_x = 1
v0_y = 2
v0_z = 3
rho0 = 1.225
c0 = 343
source2 = monopole, 1,2,3, 0.5, 10,1500,0,0.01
source10 = dipole, 0,0,0, 0.2, 1,100,0.5,1
source1 = quadrupole, 0,0,0, 0.4, 2,200,0,1
initialCondtition1 = gaussian, 6.5,6.5,1.8,1,0.05
initialCondition2 = gaussian, 0,0,0,1,1
saveFile=data.msh
precision = fp32
fluxSign = upwind
"""


def mesh():
    return D.Mesh.box_tri(2, 2, order=1, side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))


def test_parse_quirks(tmp_path):
    p = tmp_path / "c.conf"
    p.write_text(CONF)
    m = mesh()
    c = D.Config.parse(p, m)
    assert (c.time_start, c.time_end, c.time_step, c.time_rate) == (0.0, 0.2, 1e-5, 1e-4)
    assert c.num_threads == 0  # numThreads == 1 -> 0 (configParser.cpp:58)
    assert c.v0 == (1.0, 2.0, 3.0) and c.c0 == 343.0 and c.rho0 == 1.225
    assert c.time_int_method == "Runge-Kutta" and c.save_file == "data.msh"
    # std::map key order: source1 < source10 < source2
    s = c.sources
    assert s.shape == (4 + 2 + 1, 9)
    assert np.allclose(s[0], [2, -0.4, 0, 0, 0.2, 2, 200, 0, 1])          # quadrupole 1/4
    assert np.allclose(s[2], [2, 0, -0.4, 0, 0.2, 2, 200, np.pi, 1])      # quadrupole 3/4
    assert np.allclose(s[4], [1, -0.2, 0, 0, 0.1, 1, 100, 0.5, 1])        # dipole 1/2
    assert np.allclose(s[5], [1, 0.2, 0, 0, 0.1, 1, 100, 0.5 + np.pi, 1])
    assert np.allclose(s[6], [0, 1, 2, 3, 0.5, 10, 1500, 0, 0.01])        # monopole
    # only the misspelt prefix is an initial condition
    assert c.ics.shape == (1, 6) and np.allclose(c.ics[0], [0, 6.5, 6.5, 1.8, 1, 0.05])
    names = dict(zip(m.raw()["phys_name"], m.raw()["phys_tag"]))
    assert sorted(c.bcs) == sorted([(int(names["Reflecting"]), True), (int(names["Absorbing"]), False)])
    assert c.precision == "fp32" and c.flux_sign == "upwind"


def test_missing_key_is_an_error(tmp_path):
    p = tmp_path / "c.conf"
    p.write_text(CONF.replace("c0 = 343\n", ""))
    with pytest.raises(D.DGError) as e:
        D.Config.parse(p, mesh())
    assert "c0" in str(e.value)


def test_missing_file_is_an_error(tmp_path):
    with pytest.raises(D.DGError):
        D.Config.parse(tmp_path / "nope.conf", mesh())


def test_unknown_boundary_names_are_skipped(tmp_path):
    p = tmp_path / "c.conf"
    p.write_text(CONF.replace("Absorbing = Absorbing\n", ""))
    c = D.Config.parse(p, mesh())
    assert len(c.bcs) == 1 and c.bcs[0][1] is True


@pytest.mark.parametrize("step", ["0", "-1e-5", "nan", "inf"])
def test_time_step_must_advance_time(tmp_path, step):
    # the reference's loop (solver.cpp:216) would never end: refused instead
    p = tmp_path / "c.conf"
    p.write_text(CONF.replace("timeStep=1e-5\n", f"timeStep={step}\n"))
    with pytest.raises(D.DGError) as e:
        D.Config.parse(p, mesh())
    assert "timeStep" in str(e.value)
