"""Python host side of the GB300 DG acoustic RK4 library.

A thin ctypes layer over the C ABI declared in include/dgcuda.h (the GPU
solver) and include/dgmesh.h (mesh reading/generation, the reference-
semantics Mesh precompute, the .conf parser).  The flow mirrors the
reference's main (src/dgalerkin.cpp:11-63):

    mesh = Mesh.read_msh("square.msh")            # gmsh::open
    cfg = Config.parse("config.conf", mesh)       # config::parseConfig
    pre = Precomp(mesh, cfg.bcs)                  # Mesh mesh(msh, config)
    u = pre.initial_state(cfg.ics)                # Gaussian initial conditions
    sol = Solver(pre, cfg.c0, cfg.rho0, cfg.v0)   # precomputeMassMatrix + set-up
    sol.set_state(u); sol.rk4_steps(t, dt, n)     # solver::rungeKutta steps

Everything runs through lib/libdgcuda.so; there is no CPU fallback: a missing
library or a missing GPU raises DGError.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "lib" / "libdgcuda.so"

PREC_FP64, PREC_FP32, PREC_MIXED, PREC_TF32X3 = 0, 1, 2, 3
FLUX_REFERENCE, FLUX_UPWIND = 0, 1
ERRORS = {0: "ok", -1: "bad argument", -2: "CUDA error", -3: "unsupported", -4: "non-finite values",
          -5: "I/O error", -6: "mesh error", -7: "out of memory", -8: "configuration error"}


class DGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Loads lib/libdgcuda.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise DGError(-5, f"{LIB_PATH} is missing: build it with dgfem-acoustic_gb300/build.py")
        _lib = C.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


def _check_out(out, shape) -> None:
    """An output buffer the library writes into: float64, the given shape,
    every row contiguous (it is filled in place, never copied)."""
    if not isinstance(out, np.ndarray) or out.dtype != np.float64 or out.shape != shape:
        raise ValueError(f"output must be a float64 array of shape {shape}")
    if not all(out[q].flags["C_CONTIGUOUS"] for q in range(shape[0])):
        raise ValueError("output rows must be contiguous")
    if not out.flags["WRITEABLE"]:
        raise ValueError("output must be writeable")


def _check(code: int) -> None:
    if code != 0:
        raise DGError(code, lib().dg_last_error().decode(errors="replace"))


P_d, P_i, P_u8 = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_ubyte)
P_f = C.POINTER(C.c_float)


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("num_el", C.c_int), ("el_num_nodes", C.c_int),
                ("f_num", C.c_int), ("f_num_per_el", C.c_int), ("f_num_nodes", C.c_int), ("fc", C.c_int),
                ("el_jacobians", P_d), ("el_jacobian_dets", P_d), ("f_normals", P_d), ("f_jacobian_dets", P_d),
                ("el_f_ids", P_i), ("el_f_orientation", P_i), ("f_nbr_el_ids", P_i), ("f_n_to_el_n_ids", P_i),
                ("f_bc", P_i), ("f_is_boundary", P_u8),
                ("el_num_int_pts", C.c_int), ("el_int_param_coords", P_d), ("el_basis_fcts", P_d),
                ("el_ugrad_basis_fcts", P_d), ("el_jacobians_qp", P_d), ("el_jacobian_dets_qp", P_d),
                ("f_num_int_pts", C.c_int), ("f_int_param_coords", P_d), ("f_basis_fcts", P_d),
                ("f_normals_qp", P_d), ("f_jacobian_dets_qp", P_d)]


class PhysDesc(C.Structure):
    _fields_ = [("c0", C.c_double), ("rho0", C.c_double), ("v0", C.c_double * 3)]


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("flux_sign", C.c_int), ("device", C.c_int), ("use_graph", C.c_int),
                ("elems_per_block", C.c_int), ("tc_pipelines", C.c_int), ("reserved", C.c_int * 2)]


class KernelTimes(C.Structure):
    _fields_ = [("stage_ms", C.c_double * 4), ("stage_launches", C.c_int * 4), ("inject_ms", C.c_double),
                ("inject_launches", C.c_int), ("total_ms", C.c_double), ("curved_ms", C.c_double),
                ("curved_launches", C.c_int)]


class LayoutView(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("np", C.c_int), ("nf", C.c_int), ("nfp", C.c_int),
                ("nq", C.c_int), ("nperm", C.c_int), ("num_el", C.c_int), ("geo", P_d), ("fgeo", P_d),
                ("conn", P_i), ("ops", P_d), ("n_ops", C.c_int), ("tabs", P_u8), ("n_tabs", C.c_int),
                ("mass", P_d)]


class DeviceLayout(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("num_el", C.c_int), ("c0", C.c_double),
                ("rho0", C.c_double), ("v0", C.c_double * 3), ("geo", C.c_void_p), ("fgeo", C.c_void_p),
                ("conn", C.c_void_p), ("ops", C.c_void_p), ("tabs", C.c_void_p)]


class RawView(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("el_type", C.c_int), ("np", C.c_int),
                ("num_nodes", C.c_int), ("node_tags", P_i), ("xyz", P_d), ("num_el", C.c_int),
                ("el_tags", P_i), ("el_nodes", P_i), ("num_phys", C.c_int), ("phys_dim", P_i),
                ("phys_tag", P_i), ("phys_name", C.POINTER(C.c_char_p)), ("phys_node_offsets", P_i),
                ("phys_nodes", P_i)]


class ConfigView(C.Structure):
    _fields_ = [("time_start", C.c_double), ("time_end", C.c_double), ("time_step", C.c_double),
                ("time_rate", C.c_double), ("num_threads", C.c_int), ("v0", C.c_double * 3),
                ("rho0", C.c_double), ("c0", C.c_double), ("num_sources", C.c_int), ("sources", P_d),
                ("num_ics", C.c_int), ("ics", P_d), ("num_bcs", C.c_int), ("bc_phys_tags", P_i),
                ("bc_reflecting", P_i), ("element_type", C.c_char_p), ("time_int_method", C.c_char_p),
                ("save_file", C.c_char_p), ("precision", C.c_char_p), ("flux_sign", C.c_char_p)]


def _declare(L: C.CDLL) -> None:
    vp = C.c_void_p
    sig = {
        "dg_last_error": (C.c_char_p, []),
        "dg_default_opts": (None, [C.POINTER(Opts)]),
        "dg_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(PhysDesc), C.POINTER(Opts), C.POINTER(vp)]),
        "dg_destroy": (None, [vp]),
        "dg_set_state": (C.c_int, [vp, C.POINTER(P_d)]),
        "dg_get_state": (C.c_int, [vp, C.POINTER(P_d)]),
        "dg_set_sources": (C.c_int, [vp, C.c_int, P_i, P_i, P_d]),
        "dg_rk4_steps": (C.c_int, [vp, P_d, C.c_double, C.c_int]),
        "dg_rk4_steps_timed": (C.c_int, [vp, P_d, C.c_double, C.c_int, P_d]),
        "dg_profile_steps": (C.c_int, [vp, P_d, C.c_double, C.c_int, C.POINTER(KernelTimes)]),
        "dg_monitors": (C.c_int, [vp, P_d, P_d, C.POINTER(C.c_longlong)]),
        "dg_error_vs": (C.c_int, [vp, C.c_int, vp, C.c_int, P_d, C.POINTER(C.c_longlong)]),
        "dg_get_state_async": (C.c_int, [vp, P_d, C.POINTER(C.c_longlong)]),
        "dg_wait_state": (C.c_int, [vp, C.c_longlong]),
        "dg_stage_state": (C.c_int, [vp, P_d, C.POINTER(C.c_longlong)]),
        "dg_commit_state": (C.c_int, [vp, C.c_longlong]),
        "dg_synchronize": (C.c_int, [vp]),
        "dg_info": (C.c_int, [vp, C.POINTER(C.c_longlong), P_i, C.POINTER(C.c_longlong)]),
        "dg_curved_info": (C.c_int, [vp, P_i, P_i, P_i]),
        "dg_tc_info": (C.c_int, [vp, P_i, P_i]),
        "dgm_set_nodes": (C.c_int, [vp, P_d]),
        "dgm_get_curved": (C.c_int, [vp, P_i, C.POINTER(P_u8)]),
        "dg_host_alloc": (vp, [C.c_ulonglong]),
        "dg_host_free": (None, [vp]),
        "dg_layout_build": (C.c_int, [C.POINTER(MeshDesc), C.c_int, C.POINTER(vp)]),
        "dg_layout_get": (C.c_int, [vp, C.POINTER(LayoutView)]),
        "dg_layout_free": (None, [vp]),
        "dg_tc_selftest": (C.c_int, [C.c_int, P_d]),
        "dg_tc_wait_selftest": (C.c_int, [C.c_int, P_i]),
        "dg_mlp_set_gemm": (C.c_int, [vp, C.c_int]),
        "dg_tc_selftest_tf32": (C.c_int, [C.c_int, P_d]),
        "dg_euler_steps": (C.c_int, [vp, P_d, C.c_double, C.c_int]),
        "dg_multi_create": (C.c_int, [C.c_int, vp, vp, C.POINTER(Opts), C.POINTER(vp)]),
        "dg_multi_destroy": (None, [vp]),
        "dg_multi_set_state": (C.c_int, [vp, C.c_int, C.POINTER(P_d)]),
        "dg_multi_get_state": (C.c_int, [vp, C.c_int, C.POINTER(P_d)]),
        "dg_multi_set_sources": (C.c_int, [vp, C.c_int, P_i, P_i, P_i, P_d, P_d]),
        "dg_multi_rk4_steps": (C.c_int, [vp, P_d, P_d, C.c_int]),
        "dg_multi_rk4_steps_timed": (C.c_int, [vp, P_d, P_d, C.c_int, P_d]),
        "dg_multi_set_config": (C.c_int, [vp, C.c_int]),
        "dg_multi_autotune": (C.c_int, [vp, P_d, C.c_int, P_i, P_d]),
        "dg_multi_info": (C.c_int, [vp, C.POINTER(C.c_longlong), P_i, P_i, P_i]),
        "dg_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint, C.c_int, C.POINTER(vp)]),
        "dg_mlp_destroy": (None, [vp]),
        "dg_mlp_num_params": (C.c_longlong, [vp]),
        "dg_mlp_get_params": (C.c_int, [vp, P_f]),
        "dg_mlp_set_params": (C.c_int, [vp, P_f]),
        "dg_mlp_forward": (C.c_int, [vp, P_f, C.c_int, P_f]),
        "dg_mlp_forward_bf16": (C.c_int, [vp, P_f, C.c_int, P_f]),
        "dg_learned_set_inference": (C.c_int, [vp, C.c_int]),
        "dg_mlp_loss_grad": (C.c_int, [vp, P_f, P_f, C.c_int, P_d, P_f]),
        "dg_mlp_train_step": (C.c_int, [vp, P_f, P_f, C.c_int, C.c_double, P_d]),
        "dg_learned_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(PhysDesc), C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_double, C.c_uint, C.c_int, C.POINTER(vp)]),
        "dg_learned_destroy": (None, [vp]),
        "dg_learned_info": (C.c_int, [vp, P_i, P_i, C.POINTER(vp)]),
        "dg_learned_collect": (C.c_int, [vp, C.POINTER(P_d), C.c_int, C.c_int]),
        "dg_learned_num_samples": (C.c_longlong, [vp]),
        "dg_learned_train": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, C.c_uint, P_d]),
        "dg_learned_apply": (C.c_int, [vp, C.POINTER(P_d), C.c_int]),
        "dg_learned_step_stats": (C.c_int, [vp, C.POINTER(C.c_longlong), P_d, P_d]),
        "dg_parareal": (C.c_int, [vp, C.POINTER(MeshDesc), C.POINTER(PhysDesc), C.c_int, C.POINTER(P_d), C.c_int,
                                  C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(P_d), P_i, P_d]),
        "dg_create_batch": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(PhysDesc), C.POINTER(Opts), C.c_int,
                                      C.POINTER(vp)]),
        "dg_set_state_member": (C.c_int, [vp, C.c_int, C.POINTER(P_d)]),
        "dg_get_state_member": (C.c_int, [vp, C.c_int, C.POINTER(P_d)]),
        "dg_set_batch_sources": (C.c_int, [vp, C.c_int, P_i, P_i, P_i, P_d, P_d]),
        "dg_set_receivers": (C.c_int, [vp, C.c_int, P_i, C.c_int]),
        "dg_get_traces": (C.c_int, [vp, P_d, C.POINTER(C.c_int)]),
        "dg_rk4_steps_noalloc": (C.c_int, [C.POINTER(DeviceLayout), C.c_void_p, P_d, C.c_double, C.c_int,
                                           C.c_void_p]),
        "dgm_read_msh": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
        "dgm_write_msh": (C.c_int, [vp, C.c_char_p]),
        "dgm_box_tri": (C.c_int, [C.c_int, C.c_int, P_d, P_d, C.c_int, C.POINTER(C.c_char_p), C.POINTER(vp)]),
        "dgm_box_tet": (C.c_int, [C.c_int, C.c_int, C.c_int, P_d, P_d, C.c_int, C.POINTER(C.c_char_p), P_i,
                                  C.c_int, C.c_char_p, C.POINTER(vp)]),
        "dgm_get_raw": (C.c_int, [vp, C.POINTER(RawView)]),
        "dgm_free_mesh": (None, [vp]),
        "dgm_precompute": (C.c_int, [vp, C.c_int, P_i, P_i, C.POINTER(vp)]),
        "dgm_get_desc": (C.c_int, [vp, C.POINTER(MeshDesc)]),
        "dgm_get_dof_coords": (C.c_int, [vp, C.POINTER(P_d)]),
        "dgm_get_face_node_tags": (C.c_int, [vp, C.POINTER(P_i)]),
        "dgm_min_edge": (C.c_double, [vp]),
        "dgm_free_precomp": (None, [vp]),
        "dgm_gaussian_ic": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, P_d]),
        "dgm_source_dofs": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, C.c_double, P_i, C.c_int, P_i]),
        "dgm_parse_config": (C.c_int, [C.c_char_p, vp, C.POINTER(vp)]),
        "dgm_get_config": (C.c_int, [vp, C.POINTER(ConfigView)]),
        "dgm_free_config": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def pinned_array(shape) -> np.ndarray:
    """A float64 array in pinned host memory (dg_host_alloc), released with
    dg_host_free when the array is garbage collected: the buffer to give
    Solver.get_state_async for the copy to overlap the next steps."""
    import weakref

    n = int(np.prod(shape))
    p = lib().dg_host_alloc(n * 8)
    if not p:
        raise DGError(-7, lib().dg_last_error().decode(errors="replace"))
    buf = (C.c_double * n).from_address(p)
    weakref.finalize(buf, lib().dg_host_free, C.c_void_p(p))
    return np.ctypeslib.as_array(buf).reshape(shape)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(P_d)


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(P_i)


def _arr(ptr, n, dtype) -> np.ndarray:
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Mesh:
    """Raw mesh: nodes, volume elements (gmsh order) and physical groups."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dgm_free_mesh(self._h)
            self._h = None

    @classmethod
    def read_msh(cls, path: str | os.PathLike) -> "Mesh":
        h = C.c_void_p()
        _check(lib().dgm_read_msh(str(path).encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def box_tri(cls, nx: int, ny: int, lo=(-1.0, -1.0), hi=(1.0, 1.0), order: int = 3,
                side_names=("Reflecting",) * 4) -> "Mesh":
        h = C.c_void_p()
        names = (C.c_char_p * 4)(*[(s.encode() if s else None) for s in side_names])
        lo_a, hi_a = np.array(lo, float), np.array(hi, float)
        _check(lib().dgm_box_tri(nx, ny, _dptr(lo_a), _dptr(hi_a), order, names, C.byref(h)))
        return cls(h)

    @classmethod
    def box_tet(cls, nx: int, ny: int, nz: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), order: int = 3,
                side_names=("Absorbing",) * 6, removed=(), obstacle_name: str = "Reflecting") -> "Mesh":
        h = C.c_void_p()
        names = (C.c_char_p * 6)(*[(s.encode() if s else None) for s in side_names])
        lo_a, hi_a = np.array(lo, float), np.array(hi, float)
        rem = np.array(list(removed), dtype=np.int32)
        _check(lib().dgm_box_tet(nx, ny, nz, _dptr(lo_a), _dptr(hi_a), order, names,
                                 _iptr(rem) if rem.size else None, int(rem.size), obstacle_name.encode(), C.byref(h)))
        return cls(h)

    def write_msh(self, path: str | os.PathLike) -> None:
        _check(lib().dgm_write_msh(self._h, str(path).encode()))

    def set_nodes(self, xyz: np.ndarray) -> None:
        """Replace every node's coordinates (rows in node_tags order)."""
        a = np.ascontiguousarray(xyz, dtype=np.float64)
        if a.shape != (self.raw()["node_tags"].size, 3):
            raise ValueError("xyz must be [num_nodes][3]")
        _check(lib().dgm_set_nodes(self._h, _dptr(a)))

    def warp(self, fn) -> "Mesh":
        """Move every node by fn(xyz) -> xyz' (rows of [num_nodes][3]); a
        smooth nonlinear fn curves the elements.  Returns self."""
        self.set_nodes(fn(self.raw()["xyz"].copy()))
        return self

    def raw(self) -> dict:
        v = RawView()
        _check(lib().dgm_get_raw(self._h, C.byref(v)))
        off = _arr(v.phys_node_offsets, v.num_phys + 1, np.int32)
        return {
            "dim": v.dim, "order": v.order, "el_type": v.el_type, "np": v.np,
            "node_tags": _arr(v.node_tags, v.num_nodes, np.int32),
            "xyz": _arr(v.xyz, 3 * v.num_nodes, np.float64).reshape(-1, 3),
            "el_tags": _arr(v.el_tags, v.num_el, np.int32),
            "el_nodes": _arr(v.el_nodes, v.num_el * v.np, np.int32).reshape(-1, v.np),
            "phys_dim": _arr(v.phys_dim, v.num_phys, np.int32),
            "phys_tag": _arr(v.phys_tag, v.num_phys, np.int32),
            "phys_name": [v.phys_name[i].decode(errors="replace") for i in range(v.num_phys)],
            "phys_offsets": off,
            "phys_nodes": _arr(v.phys_nodes, int(off[-1]) if off.size else 0, np.int32),
        }

    def bcs(self, mapping: dict[str, bool] | None = None) -> list[tuple[int, bool]]:
        """(physical tag, reflecting) for boundary groups whose name starts with
        Reflecting/Absorbing, or as given by mapping name -> reflecting."""
        r = self.raw()
        out = []
        for d, t, n in zip(r["phys_dim"], r["phys_tag"], r["phys_name"]):
            if d != r["dim"] - 1:
                continue
            if mapping is not None:
                if n in mapping:
                    out.append((int(t), bool(mapping[n])))
            elif n.startswith("Reflecting"):
                out.append((int(t), True))
            elif n.startswith("Absorbing"):
                out.append((int(t), False))
        return sorted(out)


class Config:
    """Parsed .conf (config::parseConfig)."""

    def __init__(self, handle):
        self._h = handle
        v = ConfigView()
        _check(lib().dgm_get_config(self._h, C.byref(v)))
        self.time_start, self.time_end, self.time_step, self.time_rate = (v.time_start, v.time_end,
                                                                          v.time_step, v.time_rate)
        self.num_threads = v.num_threads
        self.v0 = tuple(v.v0)
        self.rho0, self.c0 = v.rho0, v.c0
        self.sources = _arr(v.sources, 9 * v.num_sources, np.float64).reshape(-1, 9)
        self.ics = _arr(v.ics, 6 * v.num_ics, np.float64).reshape(-1, 6)
        tags = _arr(v.bc_phys_tags, v.num_bcs, np.int32)
        refl = _arr(v.bc_reflecting, v.num_bcs, np.int32)
        self.bcs = [(int(a), bool(b)) for a, b in zip(tags, refl)]
        self.element_type = v.element_type.decode(errors="replace")
        self.time_int_method = v.time_int_method.decode(errors="replace")
        self.save_file = v.save_file.decode(errors="replace")
        self.precision = v.precision.decode(errors="replace")
        self.flux_sign = v.flux_sign.decode(errors="replace")

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dgm_free_config(self._h)
            self._h = None

    @classmethod
    def parse(cls, path: str | os.PathLike, mesh: Mesh) -> "Config":
        h = C.c_void_p()
        _check(lib().dgm_parse_config(str(path).encode(), mesh._h, C.byref(h)))
        return cls(h)


class Precomp:
    """Reference-semantics Mesh precompute (the arrays of include/Mesh.h)."""

    def __init__(self, mesh: Mesh, bcs: list[tuple[int, bool]] | None = None):
        if bcs is None:
            bcs = mesh.bcs()
        tags = np.array([b[0] for b in bcs], dtype=np.int32)
        refl = np.array([1 if b[1] else 0 for b in bcs], dtype=np.int32)
        h = C.c_void_p()
        _check(lib().dgm_precompute(mesh._h, len(bcs), _iptr(tags) if len(bcs) else None,
                                    _iptr(refl) if len(bcs) else None, C.byref(h)))
        self._h = h
        self.mesh = mesh
        d = self.desc()
        self.dim, self.order, self.num_el, self.np = d.dim, d.order, d.num_el, d.el_num_nodes
        self.f_num, self.nf, self.nfp, self.fc = d.f_num, d.f_num_per_el, d.f_num_nodes, d.fc
        self.ndof = self.num_el * self.np
        n = C.c_int()
        _check(lib().dgm_get_curved(self._h, C.byref(n), None))
        self.num_curved = n.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dgm_free_precomp(self._h)
            self._h = None

    def desc(self) -> MeshDesc:
        d = MeshDesc()
        _check(lib().dgm_get_desc(self._h, C.byref(d)))
        return d

    def arrays(self) -> dict:
        d = self.desc()
        K, F, nf, nfp = d.num_el, d.f_num, d.f_num_per_el, d.f_num_nodes
        tags = P_i()
        _check(lib().dgm_get_face_node_tags(self._h, C.byref(tags)))
        return {
            "fc": d.fc,
            "el_jacobians": _arr(d.el_jacobians, 9 * K, np.float64).reshape(K, 9),
            "el_jacobian_dets": _arr(d.el_jacobian_dets, K, np.float64),
            "f_normals": _arr(d.f_normals, 3 * F, np.float64).reshape(F, 3),
            "f_jacobian_dets": _arr(d.f_jacobian_dets, F, np.float64),
            "el_f_ids": _arr(d.el_f_ids, K * nf, np.int32).reshape(K, nf),
            "el_f_orientation": _arr(d.el_f_orientation, K * nf, np.int32).reshape(K, nf),
            "f_nbr_el_ids": _arr(d.f_nbr_el_ids, 2 * F, np.int32).reshape(F, 2),
            "f_n_to_el_n_ids": _arr(d.f_n_to_el_n_ids, 2 * F * nfp, np.int32).reshape(F, nfp, 2),
            "f_bc": _arr(d.f_bc, F, np.int32),
            "f_is_boundary": _arr(d.f_is_boundary, F, np.uint8),
            "f_node_tags": _arr(tags, F * nfp, np.int32).reshape(F, nfp),
        }

    def curved_arrays(self) -> dict:
        """Per-point arrays of a mesh with curved elements (empty otherwise)."""
        d = self.desc()
        if d.el_num_int_pts <= 0:
            return {}
        K, F, np_, nfp, ng, ngf = d.num_el, d.f_num, d.el_num_nodes, d.f_num_nodes, d.el_num_int_pts, d.f_num_int_pts
        flags = P_u8()
        n = C.c_int()
        _check(lib().dgm_get_curved(self._h, C.byref(n), C.byref(flags)))
        return {
            "curved": _arr(flags, K, np.uint8).astype(bool),
            "el_qp": _arr(d.el_int_param_coords, 4 * ng, np.float64).reshape(ng, 4),
            "el_phi": _arr(d.el_basis_fcts, ng * np_, np.float64).reshape(ng, np_),
            "el_dphi": _arr(d.el_ugrad_basis_fcts, ng * np_ * 3, np.float64).reshape(ng, np_, 3),
            "el_jac": _arr(d.el_jacobians_qp, K * ng * 9, np.float64).reshape(K, ng, 9),
            "el_detj": _arr(d.el_jacobian_dets_qp, K * ng, np.float64).reshape(K, ng),
            "f_qp": _arr(d.f_int_param_coords, 4 * ngf, np.float64).reshape(ngf, 4),
            "f_phi": _arr(d.f_basis_fcts, ngf * nfp, np.float64).reshape(ngf, nfp),
            "f_normal": _arr(d.f_normals_qp, F * ngf * 3, np.float64).reshape(F, ngf, 3),
            "f_detj": _arr(d.f_jacobian_dets_qp, F * ngf, np.float64).reshape(F, ngf),
        }

    def layout(self, flux: str = "reference") -> dict:
        """The element-centric arrays dg_create uploads (host side, no GPU)."""
        d = self.desc()
        h = C.c_void_p()
        _check(lib().dg_layout_build(C.byref(d), {"reference": FLUX_REFERENCE, "upwind": FLUX_UPWIND}[flux],
                                     C.byref(h)))
        try:
            v = LayoutView()
            _check(lib().dg_layout_get(h, C.byref(v)))
            K, nf, np_, dim = v.num_el, v.nf, v.np, v.dim
            return {
                "dim": dim, "order": v.order, "np": np_, "nf": nf, "nfp": v.nfp, "nq": v.nq, "nperm": v.nperm,
                "geo": _arr(v.geo, K * dim * dim, np.float64).reshape(K, dim, dim),
                "fgeo": _arr(v.fgeo, K * nf * 4, np.float64).reshape(K, nf, 4),
                "conn": _arr(v.conn, K * nf * 2, np.int32).reshape(K, nf, 2),
                "ops": _arr(v.ops, v.n_ops, np.float64),
                "tabs": _arr(v.tabs, v.n_tabs, np.int32),
                "mass": _arr(v.mass, np_ * np_, np.float64).reshape(np_, np_),
            }
        finally:
            lib().dg_layout_free(h)

    def dof_coords(self) -> np.ndarray:
        p = P_d()
        _check(lib().dgm_get_dof_coords(self._h, C.byref(p)))
        return _arr(p, 3 * self.ndof, np.float64).reshape(-1, 3)

    def min_edge(self) -> float:
        return float(lib().dgm_min_edge(self._h))

    def initial_state(self, ics) -> np.ndarray:
        """u[4][ndof] with the reference's Gaussian initial conditions
        (rows: 0, x, y, z, size, amp)."""
        u = np.zeros((4, self.ndof))
        for ic in ics:
            _check(lib().dgm_gaussian_ic(self._h, ic[1], ic[2], ic[3], ic[4], ic[5], _dptr(u[0])))
        return u

    def source_dofs(self, x: float, y: float, z: float, size: float) -> np.ndarray:
        cnt = C.c_int()
        _check(lib().dgm_source_dofs(self._h, x, y, z, size, None, 0, C.byref(cnt)))
        idx = np.zeros(max(cnt.value, 1), dtype=np.int32)
        _check(lib().dgm_source_dofs(self._h, x, y, z, size, _iptr(idx), cnt.value, C.byref(cnt)))
        return idx[:cnt.value]

    def gaussian_source(self, x: float, y: float, z: float, sigma: float) -> tuple[np.ndarray, np.ndarray]:
        """Nodes within 3 sigma of (x, y, z) and their weights exp(-r^2/(2 sigma^2))
        (a Gaussian-in-space hard source for dg_set_batch_sources)."""
        c = self.dof_coords()
        r2 = (c[:, 0] - x) ** 2 + (c[:, 1] - y) ** 2 + (c[:, 2] - z) ** 2
        idx = np.nonzero(r2 < (3.0 * sigma) ** 2)[0].astype(np.int32)
        return idx, np.exp(-r2[idx] / (2 * sigma * sigma))


class Solver:
    """GPU RK4 right-hand side context (dg_create ... dg_destroy)."""

    def __init__(self, pre: Precomp, c0: float, rho0: float, v0=(0.0, 0.0, 0.0), precision: str = "fp64",
                 flux: str = "reference", use_graph: bool = True, device: int = 0, nbatch: int = 1,
                 tc_pipelines: int = 0):
        d = pre.desc()
        ph = PhysDesc(c0, rho0, (C.c_double * 3)(*v0))
        o = Opts()
        lib().dg_default_opts(C.byref(o))
        o.precision = {"fp64": PREC_FP64, "fp32": PREC_FP32, "mixed": PREC_MIXED, "tf32x3": PREC_TF32X3}[precision]
        o.flux_sign = {"reference": FLUX_REFERENCE, "upwind": FLUX_UPWIND}[flux]
        o.use_graph = 1 if use_graph else 0
        o.device = device
        o.tc_pipelines = tc_pipelines
        h = C.c_void_p()
        _check(lib().dg_create_batch(C.byref(d), C.byref(ph), C.byref(o), nbatch, C.byref(h)))
        self._h = h
        self.nbatch = nbatch
        self._rec = (0, 0)
        self.pre = pre
        self.dim = pre.dim
        self.ndof = pre.ndof
        self.precision = precision

    def close(self) -> None:
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dg_destroy(self._h)
            self._h = None

    __del__ = close

    def set_state(self, u: np.ndarray, member: int | None = None) -> None:
        """Sets every batch member (member=None) or one member to u [4][ndof]."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.shape != (4, self.ndof):
            raise ValueError(f"state must have shape (4, {self.ndof}), got {u.shape}")
        ptrs = (P_d * 4)(*[_dptr(u[q]) for q in range(4)])
        if member is None:
            _check(lib().dg_set_state(self._h, ptrs))
        else:
            _check(lib().dg_set_state_member(self._h, member, ptrs))

    def get_state(self, out: np.ndarray | None = None, member: int = 0) -> np.ndarray:
        if out is None:
            out = np.empty((4, self.ndof))
        else:
            _check_out(out, (4, self.ndof))
        ptrs = (P_d * 4)(*[_dptr(out[q]) for q in range(4)])
        _check(lib().dg_get_state_member(self._h, member, ptrs))
        return out

    def set_sources(self, sources: list[tuple[np.ndarray, float, float, float, float]]) -> None:
        """sources: (dof indices, amp, freq, phase, duration) in config order."""
        off = np.zeros(len(sources) + 1, dtype=np.int32)
        idx, par = [], []
        for s, (dofs, amp, freq, phase, dur) in enumerate(sources):
            idx.append(np.asarray(dofs, dtype=np.int32))
            off[s + 1] = off[s] + len(dofs)
            par += [amp, freq, phase, dur]
        idx_a = np.concatenate(idx) if idx else np.zeros(1, dtype=np.int32)
        par_a = np.array(par if par else [0.0], dtype=np.float64)
        _check(lib().dg_set_sources(self._h, len(sources), _iptr(off), _iptr(idx_a), _dptr(par_a)))

    def set_batch_sources(self, sources: list) -> None:
        """sources: (member, dof indices, weights or None, amp, freq, phase,
        duration); source s acts on its member only."""
        n = len(sources)
        off = np.zeros(n + 1, dtype=np.int32)
        mem = np.zeros(max(n, 1), dtype=np.int32)
        idx, wts, par = [], [], []
        for s, (m, dofs, w, amp, freq, phase, dur) in enumerate(sources):
            mem[s] = m
            idx.append(np.asarray(dofs, dtype=np.int32))
            wts.append(np.ones(len(dofs)) if w is None else np.asarray(w, dtype=np.float64).reshape(-1))
            if len(wts[-1]) != len(idx[-1]):
                raise ValueError(f"source {s}: {len(idx[-1])} node indices but {len(wts[-1])} weights")
            off[s + 1] = off[s] + len(dofs)
            par += [amp, freq, phase, dur]
        idx_a = np.concatenate(idx) if idx else np.zeros(1, dtype=np.int32)
        w_a = np.concatenate(wts) if wts else np.zeros(1)
        par_a = np.array(par if par else [0.0], dtype=np.float64)
        _check(lib().dg_set_batch_sources(self._h, n, _iptr(mem), _iptr(off), _iptr(idx_a), _dptr(w_a),
                                          _dptr(par_a)))

    def set_receivers(self, dofs, max_steps: int) -> None:
        d = np.ascontiguousarray(dofs, dtype=np.int32)
        _check(lib().dg_set_receivers(self._h, len(d), _iptr(d) if len(d) else None, max_steps))
        self._rec = (len(d), max_steps)

    def traces(self) -> np.ndarray:
        """Pressure at the receivers after each recorded step: [member][rec][step]."""
        nrec, mx = self._rec
        out = np.zeros((self.nbatch, nrec, mx))
        steps = C.c_int()
        _check(lib().dg_get_traces(self._h, _dptr(out) if out.size else _dptr(np.zeros(1)), C.byref(steps)))
        return out[:, :, :steps.value]

    def rk4_steps(self, t: float, dt: float, nsteps: int) -> float:
        tt = C.c_double(t)
        _check(lib().dg_rk4_steps(self._h, C.byref(tt), dt, nsteps))
        return tt.value

    def euler_steps(self, t: float, dt: float, nsteps: int) -> float:
        """Forward-Euler steps (the reference's "Euler1" integrator)."""
        tt = C.c_double(t)
        _check(lib().dg_euler_steps(self._h, C.byref(tt), dt, nsteps))
        return tt.value

    def rk4_steps_timed(self, t: float, dt: float, nsteps: int) -> tuple[float, float]:
        """Steps bracketed by CUDA events on the solver stream: (t, device ms)."""
        tt, ms = C.c_double(t), C.c_double()
        _check(lib().dg_rk4_steps_timed(self._h, C.byref(tt), dt, nsteps, C.byref(ms)))
        return tt.value, ms.value

    def profile_steps(self, t: float, dt: float, nsteps: int) -> tuple[float, dict]:
        tt = C.c_double(t)
        kt = KernelTimes()
        _check(lib().dg_profile_steps(self._h, C.byref(tt), dt, nsteps, C.byref(kt)))
        return tt.value, {"stage_ms": list(kt.stage_ms), "stage_launches": list(kt.stage_launches),
                          "inject_ms": kt.inject_ms, "inject_launches": kt.inject_launches,
                          "total_ms": kt.total_ms, "curved_ms": kt.curved_ms, "curved_launches": kt.curved_launches}

    def monitors(self) -> tuple[float, list[float], int]:
        e = C.c_double()
        l2 = (C.c_double * 4)()
        bad = C.c_longlong()
        code = lib().dg_monitors(self._h, C.byref(e), l2, C.byref(bad))
        if code not in (0, -4):
            _check(code)
        return e.value, list(l2), bad.value

    def get_state_async(self, out: np.ndarray) -> int:
        """Starts the copy-out of member 0 into out ([4][ndof] float64,
        contiguous, ideally in pinned memory: see pinned_array) and returns
        a ticket for wait_state; out must stay alive until then."""
        if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.shape == (4, self.ndof)
                and out.flags["C_CONTIGUOUS"] and out.flags["WRITEABLE"]):
            raise ValueError(f"output must be a writeable contiguous float64 array of shape (4, {self.ndof})")
        t = C.c_longlong()
        _check(lib().dg_get_state_async(self._h, _dptr(out), C.byref(t)))
        return t.value

    def wait_state(self, ticket: int) -> None:
        _check(lib().dg_wait_state(self._h, ticket))

    def stage_state(self, u: np.ndarray) -> int:
        """Starts the upload of u ([4][ndof] float64, contiguous, ideally in
        pinned memory: see pinned_array) into a staging buffer and returns a
        ticket for commit_state; u must stay unchanged until the commit has
        run (a later step or synchronize returns after it)."""
        if not (isinstance(u, np.ndarray) and u.dtype == np.float64 and u.shape == (4, self.ndof)
                and u.flags["C_CONTIGUOUS"]):
            raise ValueError(f"state must be a contiguous float64 array of shape (4, {self.ndof})")
        t = C.c_longlong()
        _check(lib().dg_stage_state(self._h, _dptr(u), C.byref(t)))
        return t.value

    def commit_state(self, ticket: int) -> None:
        """Makes a staged state the state of member 0, after the work already
        enqueued and before any later work."""
        _check(lib().dg_commit_state(self._h, ticket))

    def error_vs(self, ref: "Solver", member: int = 0, ref_member: int = 0) -> tuple[list[float], int]:
        """FP64 relative L2 error per field of this context's state (batch
        member `member`) against `ref`'s (member `ref_member`), computed on the
        device (dg_error_vs); also the number of non-finite values."""
        rel = (C.c_double * 4)()
        bad = C.c_longlong()
        code = lib().dg_error_vs(self._h, member, ref._h, ref_member, rel, C.byref(bad))
        if code not in (0, -4):
            _check(code)
        return list(rel), bad.value

    def synchronize(self) -> None:
        _check(lib().dg_synchronize(self._h))

    def info(self) -> dict:
        d, f, b = C.c_longlong(), C.c_int(), C.c_longlong()
        _check(lib().dg_info(self._h, C.byref(d), C.byref(f), C.byref(b)))
        nc, ng, ngf = C.c_int(), C.c_int(), C.c_int()
        _check(lib().dg_curved_info(self._h, C.byref(nc), C.byref(ng), C.byref(ngf)))
        tp, te = C.c_int(), C.c_int()
        _check(lib().dg_tc_info(self._h, C.byref(tp), C.byref(te)))
        return {"dofs_per_field": d.value, "fields": f.value, "state_bytes": b.value, "curved": nc.value,
                "curved_points": ng.value, "curved_face_points": ngf.value, "tc_pipelines": tp.value,
                "tc_tile_elems": te.value}


def min_inradius(pre: Precomp) -> float:
    """Smallest inscribed radius over the elements (from the vertex nodes)."""
    x = pre.dof_coords().reshape(pre.num_el, pre.np, 3)[:, :pre.dim + 1, :]
    if pre.dim == 2:
        a = x[:, 1] - x[:, 0]
        b = x[:, 2] - x[:, 0]
        area = 0.5 * np.linalg.norm(np.cross(a, b), axis=1)
        per = (np.linalg.norm(a, axis=1) + np.linalg.norm(b, axis=1) + np.linalg.norm(x[:, 2] - x[:, 1], axis=1))
        return float(np.min(2 * area / per))
    a, b, c = x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]
    vol = np.abs(np.einsum("ij,ij->i", a, np.cross(b, c))) / 6
    faces = [(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)]
    surf = sum(0.5 * np.linalg.norm(np.cross(x[:, j] - x[:, i], x[:, k] - x[:, i]), axis=1) for i, j, k in faces)
    return float(np.min(3 * vol / surf))


def cfl_dt(pre: Precomp, c0: float, v0=(0.0, 0.0, 0.0), cfl: float = 0.5) -> float:
    """dt = CFL * h_min / ((2p+1) (c0 + |v0|)) with h_min twice the smallest
    inscribed radius (the reference takes dt from the .conf file; this is the
    rule used for the generated benchmark configurations)."""
    vmag = float(np.linalg.norm(v0))
    return cfl * 2 * min_inradius(pre) / ((2 * pre.order + 1) * (c0 + vmag))


class MultiSolver:
    """Uneven multi-mesh batch (dg_multi_*): 3D meshes of any sizes and orders
    stepped together, one persistent launch per RK4 stage."""

    def __init__(self, pres: list, phys: list, precision: str = "fp32", flux: str = "reference",
                 use_graph: bool = True, device: int = 0):
        n = len(pres)
        self._descs = (MeshDesc * n)(*[p.desc() for p in pres])
        self._phys = (PhysDesc * n)(*[PhysDesc(c0, rho0, (C.c_double * 3)(*v0)) for (c0, rho0, v0) in phys])
        o = Opts()
        lib().dg_default_opts(C.byref(o))
        o.precision = {"fp64": PREC_FP64, "fp32": PREC_FP32}[precision]
        o.flux_sign = {"reference": FLUX_REFERENCE, "upwind": FLUX_UPWIND}[flux]
        o.use_graph = 1 if use_graph else 0
        o.device = device
        h = C.c_void_p()
        _check(lib().dg_multi_create(n, C.cast(self._descs, C.c_void_p), C.cast(self._phys, C.c_void_p),
                                     C.byref(o), C.byref(h)))
        self._h = h
        self.pres = pres
        self.n = n

    def close(self) -> None:
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dg_multi_destroy(self._h)
            self._h = None

    __del__ = close

    def set_state(self, mesh: int, u: np.ndarray) -> None:
        if not 0 <= mesh < len(self.pres):
            raise ValueError(f"mesh index {mesh} out of range")
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.shape != (4, self.pres[mesh].ndof):
            raise ValueError(f"state must have shape (4, {self.pres[mesh].ndof}), got {u.shape}")
        ptrs = (P_d * 4)(*[_dptr(u[q]) for q in range(4)])
        _check(lib().dg_multi_set_state(self._h, mesh, ptrs))

    def get_state(self, mesh: int) -> np.ndarray:
        if not 0 <= mesh < len(self.pres):
            raise ValueError(f"mesh index {mesh} out of range")
        out = np.empty((4, self.pres[mesh].ndof))
        ptrs = (P_d * 4)(*[_dptr(out[q]) for q in range(4)])
        _check(lib().dg_multi_get_state(self._h, mesh, ptrs))
        return out

    def set_sources(self, sources: list) -> None:
        """sources: (mesh, dof indices, weights or None, amp, freq, phase, duration)."""
        n = len(sources)
        off = np.zeros(n + 1, dtype=np.int32)
        mesh = np.zeros(max(n, 1), dtype=np.int32)
        idx, wts, par = [], [], []
        for s, (m, dofs, w, amp, freq, phase, dur) in enumerate(sources):
            mesh[s] = m
            idx.append(np.asarray(dofs, dtype=np.int32))
            wts.append(np.ones(len(dofs)) if w is None else np.asarray(w, dtype=np.float64).reshape(-1))
            if len(wts[-1]) != len(idx[-1]):
                raise ValueError(f"source {s}: {len(idx[-1])} node indices but {len(wts[-1])} weights")
            off[s + 1] = off[s] + len(dofs)
            par += [amp, freq, phase, dur]
        idx_a = np.concatenate(idx) if idx else np.zeros(1, dtype=np.int32)
        w_a = np.concatenate(wts) if wts else np.zeros(1)
        par_a = np.array(par if par else [0.0], dtype=np.float64)
        _check(lib().dg_multi_set_sources(self._h, n, _iptr(mesh), _iptr(off), _iptr(idx_a), _dptr(w_a),
                                          _dptr(par_a)))

    def _per_mesh(self, a, name: str) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        if a.size != len(self.pres):
            raise ValueError(f"{name} needs one value per mesh ({len(self.pres)}), got {a.size}")
        return a

    def rk4_steps(self, t, dt, nsteps: int) -> np.ndarray:
        tt = self._per_mesh(t, "t").copy()
        d = self._per_mesh(dt, "dt")
        _check(lib().dg_multi_rk4_steps(self._h, _dptr(tt), _dptr(d), nsteps))
        return tt

    def rk4_steps_timed(self, t, dt, nsteps: int) -> tuple[np.ndarray, float]:
        tt = self._per_mesh(t, "t").copy()
        d = self._per_mesh(dt, "dt")
        ms = C.c_double()
        _check(lib().dg_multi_rk4_steps_timed(self._h, _dptr(tt), _dptr(d), nsteps, C.byref(ms)))
        return tt, ms.value

    def set_config(self, cfg: int) -> None:
        _check(lib().dg_multi_set_config(self._h, cfg))

    def autotune(self, dt, trial_steps: int = 4) -> tuple[int, list]:
        d = self._per_mesh(dt, "dt")
        info = self.info()
        ms = np.zeros(info["ncfg"])
        ch = C.c_int()
        _check(lib().dg_multi_autotune(self._h, _dptr(d), trial_steps, C.byref(ch), _dptr(ms)))
        return ch.value, ms.tolist()

    def info(self) -> dict:
        dofs = C.c_longlong()
        ncfg, cfg = C.c_int(), C.c_int()
        bt = (C.c_int * 8)()
        _check(lib().dg_multi_info(self._h, C.byref(dofs), C.byref(ncfg), C.byref(cfg), bt))
        return {"dofs_per_field": dofs.value, "ncfg": ncfg.value, "cfg": cfg.value,
                "block_threads": list(bt)[:ncfg.value]}


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(P_f)


class MLP:
    """dg_mlp: FP32 MLP nin -> width (GELU) x hidden_layers -> nout, trained
    on the GPU by the library's own kernels."""

    def __init__(self, nin: int, width: int, nout: int, hidden_layers: int, seed: int = 0, device: int = 0):
        h = C.c_void_p()
        _check(lib().dg_mlp_create(nin, width, nout, hidden_layers, seed, device, C.byref(h)))
        self._h = h
        self.nin, self.width, self.nout, self.hidden = nin, width, nout, hidden_layers

    def close(self) -> None:
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dg_mlp_destroy(self._h)
            self._h = None

    __del__ = close

    def num_params(self) -> int:
        return int(lib().dg_mlp_num_params(self._h))

    def params(self) -> np.ndarray:
        p = np.zeros(self.num_params(), dtype=np.float32)
        _check(lib().dg_mlp_get_params(self._h, _fptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().dg_mlp_set_params(self._h, _fptr(p)))

    def set_gemm(self, mode: str) -> None:
        """"tc" (default): the GEMMs of training on the tensor cores with
        3xTF32 split products; "simt": on the CUDA cores.  FP32 inference
        runs on the CUDA cores either way."""
        _check(lib().dg_mlp_set_gemm(self._h, {"simt": 0, "tc": 1}[mode]))

    def forward(self, X: np.ndarray, bf16: bool = False) -> np.ndarray:
        """Inference; bf16=True runs it on the tensor cores (BF16 inputs,
        weights and hidden activations, FP32 accumulation)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.empty((X.shape[0], self.nout), dtype=np.float32)
        fn = lib().dg_mlp_forward_bf16 if bf16 else lib().dg_mlp_forward
        _check(fn(self._h, _fptr(X), X.shape[0], _fptr(Y)))
        return Y

    def loss_grad(self, X: np.ndarray, T: np.ndarray) -> tuple[float, np.ndarray]:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.num_params(), dtype=np.float32)
        loss = C.c_double()
        _check(lib().dg_mlp_loss_grad(self._h, _fptr(X), _fptr(T), X.shape[0], C.byref(loss), _fptr(g)))
        return loss.value, g

    def train_step(self, X: np.ndarray, T: np.ndarray, lr: float) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = C.c_double()
        _check(lib().dg_mlp_train_step(self._h, _fptr(X), _fptr(T), X.shape[0], lr, C.byref(loss)))
        return loss.value


class Learned:
    """dg_learned: element-local network as coarse propagator of coarse_steps
    fine RK4 steps on one mesh."""

    def __init__(self, pre: Precomp, c0: float, rho0: float, v0=(0.0, 0.0, 0.0), flux: str = "upwind",
                 width: int = 256, hidden_layers: int = 3, coarse_steps: int = 10, dt: float = 1e-6, seed: int = 0,
                 device: int = 0):
        self._desc = pre.desc()
        self._phys = PhysDesc(c0, rho0, (C.c_double * 3)(*v0))
        self.flux = {"reference": FLUX_REFERENCE, "upwind": FLUX_UPWIND}[flux]
        h = C.c_void_p()
        _check(lib().dg_learned_create(C.byref(self._desc), C.byref(self._phys), self.flux, width, hidden_layers,
                                       coarse_steps, dt, seed, device, C.byref(h)))
        self._h = h
        self.pre = pre
        self.coarse_steps = coarse_steps
        self.dt = dt

    def close(self) -> None:
        if getattr(self, "_h", None) and _lib is not None:
            _lib.dg_learned_destroy(self._h)
            self._h = None

    __del__ = close

    def collect(self, u0: np.ndarray, nsnap: int, max_rows: int = 1 << 20) -> None:
        u0 = np.ascontiguousarray(u0, dtype=np.float64)
        ptrs = (P_d * 4)(*[_dptr(u0[q]) for q in range(4)])
        _check(lib().dg_learned_collect(self._h, ptrs, nsnap, max_rows))

    def num_samples(self) -> int:
        return int(lib().dg_learned_num_samples(self._h))

    def train(self, epochs: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_double()
        _check(lib().dg_learned_train(self._h, epochs, batch, lr, seed, C.byref(loss)))
        return loss.value

    def set_inference(self, mode: str) -> None:
        """Coarse steps infer in "fp32" (default) or "bf16" (tensor cores)."""
        _check(lib().dg_learned_set_inference(self._h, {"fp32": 0, "bf16": 1}[mode]))

    def set_gemm(self, mode: str) -> None:
        """GEMMs of the network's training: "tc" (default, tensor cores,
        3xTF32) or "simt" (CUDA cores)."""
        ni, no, net = C.c_int(), C.c_int(), C.c_void_p()
        _check(lib().dg_learned_info(self._h, C.byref(ni), C.byref(no), C.byref(net)))
        _check(lib().dg_mlp_set_gemm(net, {"simt": 0, "tc": 1}[mode]))

    def step_stats(self) -> dict:
        n, am, amin = C.c_longlong(), C.c_double(), C.c_double()
        _check(lib().dg_learned_step_stats(self._h, C.byref(n), C.byref(am), C.byref(amin)))
        return {"applications": n.value, "alpha_mean": am.value, "alpha_min": amin.value}

    def apply(self, u: np.ndarray, napps: int) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        ptrs = (P_d * 4)(*[_dptr(u[q]) for q in range(4)])
        _check(lib().dg_learned_apply(self._h, ptrs, napps))
        return u


def parareal(pre: Precomp, c0: float, rho0: float, u0: np.ndarray, nslices: int, slice_steps: int, dt: float,
             tol: float, max_iter: int, learned: "Learned | None" = None, v0=(0.0, 0.0, 0.0),
             flux: str = "upwind") -> tuple[np.ndarray, int, list]:
    """dg_parareal: returns (end state of the last slice, iterations, change per iteration)."""
    desc = pre.desc()
    phys = PhysDesc(c0, rho0, (C.c_double * 3)(*v0))
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    uin = (P_d * 4)(*[_dptr(u0[q]) for q in range(4)])
    out = np.zeros_like(u0)
    uout = (P_d * 4)(*[_dptr(out[q]) for q in range(4)])
    it = C.c_int()
    hist = np.zeros(max(max_iter, 1))
    _check(lib().dg_parareal(learned._h if learned else None, C.byref(desc), C.byref(phys),
                             {"reference": FLUX_REFERENCE, "upwind": FLUX_UPWIND}[flux], uin, nslices, slice_steps, dt,
                             tol, max_iter, uout, C.byref(it), _dptr(hist)))
    return out, it.value, hist[:it.value].tolist()
