"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle
(oracle/build/liboracle.so, built by oracle/Makefile).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

P_d, P_i = C.POINTER(C.c_double), C.POINTER(C.c_int)


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


class OracleInput(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("np", C.c_int), ("num_nodes", C.c_int),
                ("node_tags", P_i), ("xyz", P_d), ("num_el", C.c_int), ("el_tags", P_i), ("el_nodes", P_i),
                ("num_groups", C.c_int), ("group_dim", P_i), ("group_tag", P_i), ("group_offsets", P_i),
                ("group_nodes", P_i), ("time_step", C.c_double), ("num_threads", C.c_int),
                ("v0", C.c_double * 3), ("rho0", C.c_double), ("c0", C.c_double), ("num_sources", C.c_int),
                ("sources", P_d), ("num_bcs", C.c_int), ("bc_tags", P_i), ("bc_reflecting", P_i),
                ("upwind", C.c_int)]


class MeshView(C.Structure):
    _fields_ = [("fc", C.c_int), ("num_el", C.c_int), ("f_num", C.c_int), ("nf", C.c_int), ("nfp", C.c_int),
                ("np", C.c_int), ("n_el_qp", C.c_int), ("n_f_qp", C.c_int), ("el_f_ids", P_i),
                ("el_f_orientation", P_i), ("f_node_tags", P_i), ("f_bc", P_i), ("el_jac_dets", P_d),
                ("f_jac_dets", P_d), ("f_normals", P_d)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(OracleInput), C.c_char_p, C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_num_dofs.argtypes = [C.c_void_p]
        L.oracle_set_state.argtypes = [C.c_void_p, P_d]
        L.oracle_get_state.argtypes = [C.c_void_p, P_d]
        L.oracle_run.argtypes = [C.c_void_p, P_d, C.c_int, C.c_int, P_d]
        L.oracle_run_until.argtypes = [C.c_void_p, C.c_double, C.c_double, P_d]
        L.oracle_mesh.argtypes = [C.c_void_p, C.POINTER(MeshView)]
        L.oracle_face_maps.argtypes = [C.c_void_p, P_i, P_i]
        L.oracle_rhs.argtypes = [C.c_void_p, P_d, P_d]
        L.oracle_set_method.argtypes = [C.c_void_p, C.c_int]
        L.oracle_reference_element.argtypes = [C.c_int, C.c_int, P_d, P_d, P_d, P_i, P_d, P_d, P_d]
        _lib = L
    return _lib


def reference_element(dim: int, order: int) -> dict:
    """The oracle's reference element of the given dimension and order: node
    lattice [n][3], Gauss(2p) rule [ng][4] (u, v, w, weight), the Lagrange
    basis and its gradients at the rule points ([ng][n], [ng][n][3]), and
    the mass and stiffness matrices that rule gives with that basis."""
    L = lib()
    ng = C.c_int()
    n = L.oracle_reference_element(dim, order, None, None, None, C.byref(ng), None, None, None)
    if n < 0:
        raise ValueError(f"no reference element for dim {dim}, order {order}")
    nodes, mass = np.empty((n, 3)), np.empty((n, n))
    stiff, rule = np.empty((dim, n, n)), np.empty((ng.value, 4))
    phi, grad = np.empty((ng.value, n)), np.empty((ng.value, n, 3))
    L.oracle_reference_element(dim, order, nodes.ctypes.data_as(P_d), mass.ctypes.data_as(P_d),
                               stiff.ctypes.data_as(P_d), C.byref(ng), rule.ctypes.data_as(P_d),
                               phi.ctypes.data_as(P_d), grad.ctypes.data_as(P_d))
    return {"nodes": nodes, "mass": mass, "stiff": stiff, "rule": rule, "phi": phi, "grad": grad}


def _arr(ptr, n, dtype):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True) if n else np.zeros(0, dtype)


class Oracle:
    """Faithful CPU restatement of the reference solver on a raw mesh.

    num_threads is the reference's numThreads configuration key: the OpenMP
    team of its element and face loops, with 0 (and 1, which the reference
    reads as 0) meaning the OpenMP default team."""

    def __init__(self, raw: dict, time_step: float, c0: float, rho0: float, v0=(0.0, 0.0, 0.0),
                 bcs=(), sources=None, num_threads: int = 0, upwind: bool = False):
        self._keep = []

        def keep(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            self._keep.append(a)
            return a

        inp = OracleInput()
        inp.dim, inp.order, inp.np = raw["dim"], raw["order"], raw["np"]
        nt = keep(raw["node_tags"], np.int32)
        xyz = keep(raw["xyz"].reshape(-1), np.float64)
        et = keep(raw["el_tags"], np.int32)
        en = keep(raw["el_nodes"].reshape(-1), np.int32)
        inp.num_nodes = nt.size
        inp.node_tags, inp.xyz = nt.ctypes.data_as(P_i), xyz.ctypes.data_as(P_d)
        inp.num_el = et.size
        inp.el_tags, inp.el_nodes = et.ctypes.data_as(P_i), en.ctypes.data_as(P_i)
        gd, gt = keep(raw["phys_dim"], np.int32), keep(raw["phys_tag"], np.int32)
        go, gn = keep(raw["phys_offsets"], np.int32), keep(raw["phys_nodes"], np.int32)
        if gn.size == 0:
            gn = keep(np.zeros(1), np.int32)
        inp.num_groups = gd.size
        inp.group_dim, inp.group_tag = gd.ctypes.data_as(P_i), gt.ctypes.data_as(P_i)
        inp.group_offsets, inp.group_nodes = go.ctypes.data_as(P_i), gn.ctypes.data_as(P_i)
        inp.time_step = time_step
        inp.num_threads = num_threads
        inp.v0 = (C.c_double * 3)(*v0)
        inp.rho0, inp.c0 = rho0, c0
        src = keep(np.zeros((0, 9)) if sources is None else np.asarray(sources).reshape(-1, 9), np.float64)
        inp.num_sources = src.shape[0]
        inp.sources = src.ctypes.data_as(P_d) if src.size else None
        bt = keep([b[0] for b in bcs] or [0], np.int32)
        br = keep([1 if b[1] else 0 for b in bcs] or [0], np.int32)
        inp.num_bcs = len(bcs)
        inp.bc_tags, inp.bc_reflecting = bt.ctypes.data_as(P_i), br.ctypes.data_as(P_i)
        inp.upwind = 1 if upwind else 0
        err = C.create_string_buffer(512)
        h = lib().oracle_create(C.byref(inp), err, 512)
        if not h:
            raise RuntimeError("oracle: " + err.value.decode())
        self._h = C.c_void_p(h)
        self.ndof = lib().oracle_num_dofs(self._h)
        self.time_step = time_step

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_destroy(self._h)
            self._h = None

    def set_state(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        if u.size != 4 * self.ndof:
            raise ValueError(f"state must hold 4 x {self.ndof} values, got {u.size}")
        lib().oracle_set_state(self._h, u.ctypes.data_as(P_d))

    def get_state(self) -> np.ndarray:
        u = np.empty(4 * self.ndof)
        lib().oracle_get_state(self._h, u.ctypes.data_as(P_d))
        return u.reshape(4, self.ndof)

    def set_method(self, method: str) -> None:
        """"Runge-Kutta" (classical RK4) or "Euler1" (forward Euler), the two
        timeIntMethod values the reference's main dispatches on."""
        code = {"Runge-Kutta": 0, "Euler1": 1}[method]
        lib().oracle_set_method(self._h, code)

    def run(self, t: float, nsteps: int, dedup: bool = False) -> tuple[float, float]:
        tt, sec = C.c_double(t), C.c_double()
        lib().oracle_run(self._h, C.byref(tt), nsteps, 1 if dedup else 0, C.byref(sec))
        return tt.value, sec.value

    def run_until(self, t_start: float, time_end: float) -> tuple[int, float]:
        sec = C.c_double()
        n = lib().oracle_run_until(self._h, t_start, time_end, C.byref(sec))
        return n, sec.value

    def rhs(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        if u.size != 4 * self.ndof:
            raise ValueError(f"state must hold 4 x {self.ndof} values, got {u.size}")
        out = np.empty_like(u)
        lib().oracle_rhs(self._h, u.ctypes.data_as(P_d), out.ctypes.data_as(P_d))
        return out.reshape(4, self.ndof)

    def mesh(self) -> dict:
        v = MeshView()
        lib().oracle_mesh(self._h, C.byref(v))
        K, F, nf, nfp = v.num_el, v.f_num, v.nf, v.nfp
        nbr = np.empty(2 * F, dtype=np.int32)
        fn = np.empty(2 * F * nfp, dtype=np.int32)
        lib().oracle_face_maps(self._h, nbr.ctypes.data_as(P_i), fn.ctypes.data_as(P_i))
        return {
            "fc": v.fc,
            "el_f_ids": _arr(v.el_f_ids, K * nf, np.int32).reshape(K, nf),
            "el_f_orientation": _arr(v.el_f_orientation, K * nf, np.int32).reshape(K, nf),
            "f_node_tags": _arr(v.f_node_tags, F * nfp, np.int32).reshape(F, nfp),
            "f_bc": _arr(v.f_bc, F, np.int32),
            "el_jacobian_dets": _arr(v.el_jac_dets, K * v.n_el_qp, np.float64).reshape(K, v.n_el_qp),
            "f_jacobian_dets": _arr(v.f_jac_dets, F * v.n_f_qp, np.float64).reshape(F, v.n_f_qp),
            "f_normals": _arr(v.f_normals, F * v.n_f_qp * 3, np.float64).reshape(F, v.n_f_qp, 3),
            "f_nbr_el_ids": nbr.reshape(F, 2),
            "f_n_to_el_n_ids": fn.reshape(F, nfp, 2),
        }
