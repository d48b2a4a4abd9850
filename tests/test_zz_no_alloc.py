"""dg_rk4_steps_noalloc: the RK4 entry point for callers that cannot allocate
device memory (an application that owns every device byte through its own
pool, time loops that cannot take the synchronisation an allocation may
cause).  The caller owns the layout and the state on the
device; the stage buffers come from a fixed array inside the library.

The test gives it device arrays it allocated itself (through torch, as such
a caller's own pool would) and compares two consecutive calls, enqueued on a
stream of the caller's own, with the allocating entry point dg_rk4_steps on
the same input, to the FP64 parity tolerance of the other GPU tests (1e-10
relative L2 per field).  Around the second call it checks the property the
entry point exists for: the device's free memory and torch's allocated
bytes do not change (the first call may load the library's device array
into the context; later calls allocate nothing)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import dgcuda as D

pytestmark = pytest.mark.gpu

TOL = 1e-10
C0, RHO0 = 340.0, 1.225


def _device_array(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to("cuda:0")


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh = D.Mesh.box_tri(6, 5, (-1.0, -1.0), (1.0, 1.0), order=3,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    pre = D.Precomp(mesh)
    v0 = (40.0, -25.0, 0.0)
    dt = D.cfl_dt(pre, C0, v0)
    nq = pre.dim + 1
    u0 = pre.initial_state([(0, 0.2, -0.1, 0.0, 0.05, 1.0)])
    u0[1:nq] += 1e-3 * np.random.default_rng(7).standard_normal((nq - 1, pre.ndof))

    # allocating entry point
    sol = D.Solver(pre, C0, RHO0, v0, precision="fp64")
    sol.set_state(u0)
    refs = []
    t = 0.0
    for _ in range(2):
        t = sol.rk4_steps(t, dt, 7)
        refs.append(sol.get_state()[:nq].copy())
    sol.close()

    # caller-owned device arrays
    lay = pre.layout("reference")
    keep = {
        "geo": _device_array(torch, lay["geo"].reshape(-1), np.float64),
        "fgeo": _device_array(torch, lay["fgeo"].reshape(-1), np.float64),
        "conn": _device_array(torch, lay["conn"].reshape(-1), np.int32),
        "ops": _device_array(torch, lay["ops"], np.float64),
        "tabs": _device_array(torch, lay["tabs"], np.uint8),
        "u": _device_array(torch, u0[:nq].reshape(-1), np.float64),
    }
    dl = D.DeviceLayout()
    dl.dim, dl.order, dl.num_el = pre.dim, pre.order, pre.num_el
    dl.c0, dl.rho0 = C0, RHO0
    dl.v0 = (C.c_double * 3)(*v0)
    for k in ("geo", "fgeo", "conn", "ops", "tabs"):
        setattr(dl, k, keep[k].data_ptr())
    tt = C.c_double(0.0)
    stream = torch.cuda.Stream()
    mem = []
    for call in range(2):
        torch.cuda.synchronize()
        mem.append((torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()))
        code = D.lib().dg_rk4_steps_noalloc(C.byref(dl), keep["u"].data_ptr(), C.byref(tt), dt, 7,
                                            C.c_void_p(stream.cuda_stream))
        assert code == 0, D.lib().dg_last_error().decode()
        stream.synchronize()
        torch.cuda.synchronize()
        if call == 1:
            assert (torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()) == mem[1]
        got = keep["u"].cpu().numpy().reshape(nq, pre.ndof)
        for q in range(nq):
            ref = refs[call][q]
            rel = np.linalg.norm(got[q] - ref) / np.linalg.norm(ref)
            assert rel <= TOL, (call, q, rel)
    assert tt.value == pytest.approx(14 * dt)
