"""The C ABI library loads and exports every function declared in include/."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import dgcuda as D

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b((?:dg|dgm)_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(str(D.LIB_PATH))
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_have_messages():
    m = D.Mesh.box_tri(2, 2, order=1)
    pre = D.Precomp(m)
    d = pre.desc()
    d.order = 9
    h = ctypes.c_void_p()
    code = D.lib().dg_layout_build(ctypes.byref(d), 0, ctypes.byref(h))
    assert code == -6
    assert b"order" in D.lib().dg_last_error()
