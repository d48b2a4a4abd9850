"""dg_create rejects bad arguments and inconsistent meshes on the host,
before any device call, with the documented error code and a message.  The
kernels index device memory through the caller's face ids, neighbour ids and
face node maps, so every such array is range-checked here.  (No GPU: a check
that were missing would reach the device calls and return DG_ERR_CUDA.)"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

import dgcuda as D

DG_ERR_ARG, DG_ERR_UNSUPPORTED, DG_ERR_MESH = -1, -3, -6


class Desc:
    """A mesh descriptor whose arrays are private copies that a test may
    corrupt."""

    def __init__(self, dim: int, order: int):
        m = D.Mesh.box_tri(2, 2, order=order) if dim == 2 else D.Mesh.box_tet(2, 2, 2, order=order)
        self.pre = D.Precomp(m)
        self.d = self.pre.desc()
        a = self.pre.arrays()
        self.a = {k: np.ascontiguousarray(v) for k, v in a.items() if isinstance(v, np.ndarray)}
        self._point()

    def _point(self):
        d, a = self.d, self.a
        d.el_jacobians = a["el_jacobians"].ctypes.data_as(D.P_d)
        d.el_jacobian_dets = a["el_jacobian_dets"].ctypes.data_as(D.P_d)
        d.f_normals = a["f_normals"].ctypes.data_as(D.P_d)
        d.f_jacobian_dets = a["f_jacobian_dets"].ctypes.data_as(D.P_d)
        d.el_f_ids = a["el_f_ids"].ctypes.data_as(D.P_i)
        d.el_f_orientation = a["el_f_orientation"].ctypes.data_as(D.P_i)
        d.f_nbr_el_ids = a["f_nbr_el_ids"].ctypes.data_as(D.P_i)
        d.f_n_to_el_n_ids = a["f_n_to_el_n_ids"].ctypes.data_as(D.P_i)
        d.f_bc = a["f_bc"].ctypes.data_as(D.P_i)
        d.f_is_boundary = a["f_is_boundary"].ctypes.data_as(D.P_u8)

    def interior_face(self) -> int:
        return int(np.flatnonzero(self.a["f_is_boundary"] == 0)[0])


def create(d, c0=340.0, rho0=1.225, precision=0, flux=0, nbatch=1, null_mesh=False):
    ph = D.PhysDesc()
    ph.c0, ph.rho0 = c0, rho0
    o = D.Opts()
    D.lib().dg_default_opts(C.byref(o))
    o.precision, o.flux_sign = precision, flux
    h = C.c_void_p()
    code = D.lib().dg_create_batch(None if null_mesh else C.byref(d), C.byref(ph), C.byref(o), nbatch, C.byref(h))
    msg = (D.lib().dg_last_error() or b"").decode()
    return code, msg, h


@pytest.mark.parametrize("dim", [2, 3])
def test_arguments(dim):
    x = Desc(dim, 2)
    assert create(x.d, null_mesh=True)[0] == DG_ERR_ARG
    for nb in (0, 65536):
        code, msg, h = create(x.d, nbatch=nb)
        assert code == DG_ERR_ARG and "batch" in msg and not h.value
    code, msg, _ = create(x.d, precision=7)
    assert code == DG_ERR_ARG and "precision" in msg
    code, msg, _ = create(x.d, flux=9)
    assert code == DG_ERR_ARG and "flux" in msg
    for c0, rho0 in ((0.0, 1.2), (340.0, -1.0), (math.nan, 1.2)):
        code, msg, _ = create(x.d, c0=c0, rho0=rho0)
        assert code == DG_ERR_ARG and "positive" in msg


def test_unsupported_dimension_and_order():
    x = Desc(3, 2)
    x.d.dim = 4
    assert create(x.d)[0] == DG_ERR_UNSUPPORTED
    x.d.dim = 3
    x.d.order = 6
    code, msg, _ = create(x.d)
    assert code == DG_ERR_UNSUPPORTED and "order" in msg


@pytest.mark.parametrize("dim", [2, 3])
def test_inconsistent_meshes(dim):
    cases = []

    def case(name, fn, words):
        cases.append((name, fn, words))

    case("empty", lambda x: setattr(x.d, "num_el", 0), "empty")
    case("node count", lambda x: setattr(x.d, "el_num_nodes", x.d.el_num_nodes + 1), "node counts")
    case("null array", lambda x: setattr(x.d, "f_normals", D.P_d()), "null")
    case("face id high", lambda x: x.a["el_f_ids"].__setitem__((0, 0), x.d.f_num), "face id out of range")
    case("face id negative", lambda x: x.a["el_f_ids"].__setitem__((1, 1), -1), "face id out of range")
    case("neighbour out of range",
         lambda x: x.a["f_nbr_el_ids"].__setitem__((x.interior_face(), 1), x.d.num_el + 5), "neighbour")
    case("face node map", lambda x: x.a["f_n_to_el_n_ids"].__setitem__((x.interior_face(), 0, 0), 10 ** 6),
         "face node map")
    case("singular Jacobian", lambda x: x.a["el_jacobians"].__setitem__(0, 0.0), "Jacobian")
    for name, fn, words in cases:
        x = Desc(dim, 2)
        fn(x)
        code, msg, h = create(x.d)
        assert code == DG_ERR_MESH, (name, code, msg)
        assert words in msg, (name, msg)
        assert not h.value


def test_last_error_is_per_thread():
    import threading

    x, y = Desc(2, 2), Desc(3, 2)
    x.d.order = 9          # -> "order must be in 1..5"
    y.d.num_el = 0         # -> "empty mesh"
    got = {}
    barrier = threading.Barrier(2)

    def work(name, d):
        barrier.wait()
        for _ in range(200):
            code, msg, _ = create(d)
            got.setdefault(name, set()).add((code, msg))

    ts = [threading.Thread(target=work, args=("order", x.d)), threading.Thread(target=work, args=("empty", y.d))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert len(got["order"]) == 1 and len(got["empty"]) == 1
    (c1, m1), = got["order"]
    (c2, m2), = got["empty"]
    assert c1 == DG_ERR_UNSUPPORTED and "order" in m1
    assert c2 == DG_ERR_MESH and "empty" in m2


def test_mesh_generators_refuse_oversized_and_negative_inputs():
    with pytest.raises(D.DGError, match="too large"):
        D.Mesh.box_tri(100000, 100000, order=5)
    with pytest.raises(D.DGError, match="too large"):
        D.Mesh.box_tet(2000, 2000, 2000, order=3)
    with pytest.raises(D.DGError):
        D.Mesh.box_tri(0, 3, order=2)
    lo, hi = (C.c_double * 3)(0, 0, 0), (C.c_double * 3)(1, 1, 1)
    removed = (C.c_int * 1)(0)
    h = C.c_void_p()
    code = D.lib().dgm_box_tet(2, 2, 2, lo, hi, 2, None, removed, -5, None, C.byref(h))
    assert code == DG_ERR_ARG and not h.value


def _fake_device_layout(dim=2, order=3, num_el=8, ptr=4096):
    dl = D.DeviceLayout()
    dl.dim, dl.order, dl.num_el = dim, order, num_el
    dl.c0, dl.rho0 = 340.0, 1.225
    for k in ("geo", "fgeo", "conn", "ops", "tabs"):
        setattr(dl, k, ptr)
    return dl


@pytest.mark.parametrize("field,value,msg", [("fgeo", 4096 + 8, b"fgeo must be 16-byte"),
                                             ("conn", 4096 + 4, b"conn must be 8-byte"),
                                             ("geo", 4096 + 4, b"8-byte"), ("ops", 4096 + 2, b"8-byte")])
def test_noalloc_refuses_misaligned_layout_pointers_before_any_launch(field, value, msg):
    """The stage kernels read fgeo as 16-byte vectors and conn as 8-byte
    pairs: dg_rk4_steps_noalloc checks the caller's pointers on the host and
    returns DG_ERR_ARG before touching the device (no GPU needed here)."""
    dl = _fake_device_layout()
    setattr(dl, field, value)
    tt = C.c_double(0.0)
    code = D.lib().dg_rk4_steps_noalloc(C.byref(dl), C.c_void_p(4096), C.byref(tt), 1e-6, 1, None)
    assert code == -1
    assert msg in D.lib().dg_last_error()
    code = D.lib().dg_rk4_steps_noalloc(C.byref(_fake_device_layout()), C.c_void_p(4096 + 4), C.byref(tt),
                                        1e-6, 1, None)
    assert code == -1 and b"u must be 8-byte" in D.lib().dg_last_error()
    assert tt.value == 0.0


def test_noalloc_rejects_states_beyond_capacity():
    dl = _fake_device_layout(dim=3, order=5, num_el=1 << 20)
    tt = C.c_double(0.0)
    code = D.lib().dg_rk4_steps_noalloc(C.byref(dl), C.c_void_p(4096), C.byref(tt), 1e-6, 1, None)
    assert code == -3
    assert b"capacity" in D.lib().dg_last_error()


def test_state_transfer_entry_points_refuse_null_arguments():
    """The overlapped state transfers check their arguments before any device
    call: a null context, host array or ticket pointer is DG_ERR_ARG with a
    message (no GPU needed)."""
    lib = D.lib()
    host = np.zeros(16)
    t = C.c_longlong()
    for code in (lib.dg_stage_state(None, host.ctypes.data_as(D.P_d), C.byref(t)),
                 lib.dg_stage_state(None, None, C.byref(t)),
                 lib.dg_commit_state(None, 0),
                 lib.dg_get_state_async(None, host.ctypes.data_as(D.P_d), C.byref(t)),
                 lib.dg_wait_state(None, 0)):
        assert code == DG_ERR_ARG
        assert lib.dg_last_error()
