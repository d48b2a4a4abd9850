"""Failure detection on the host (CPU only): a host allocation that fails
inside the library comes back as DG_ERR_NOMEM through the C ABI instead of
an exception or a crash.  The failure is forced in a child process whose
address space is capped (RLIMIT_AS) just above what it already uses, then a
mesh far larger than the cap is generated."""
from __future__ import annotations

import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = textwrap.dedent("""
    import resource, sys
    sys.path.insert(0, {pkg!r})
    import dgcuda as D
    D.lib()
    small = D.Mesh.box_tet(2, 2, 2, order=3)          # works before the cap
    with open("/proc/self/status") as f:
        vm = next(int(l.split()[1]) for l in f if l.startswith("VmSize:")) * 1024
    cap = vm + (96 << 20)
    resource.setrlimit(resource.RLIMIT_AS, (cap, cap))
    try:
        D.Mesh.box_tet(96, 96, 96, order=3)           # ~5.3 M tets: several GB
    except D.DGError as e:
        print("code", e.code)
    else:
        print("code", 0)
""")


@pytest.mark.skipif(sys.platform != "linux", reason="RLIMIT_AS and /proc are Linux features")
def test_host_allocation_failure_is_reported_as_nomem():
    code = CHILD.format(pkg=str(ROOT / "dgfem-acoustic_gb300"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "code -7" in r.stdout, (r.stdout, r.stderr[-2000:])
