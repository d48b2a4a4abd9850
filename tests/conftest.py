"""Shared test set-up: paths, build of the library and the oracle, markers."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "dgfem-acoustic_gb300"
for p in (str(PKG), str(ROOT / "oracle"), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the product kernels)")


_built = False


def _build_once():
    global _built
    if _built:
        return
    import importlib.util

    spec = importlib.util.spec_from_file_location("dgfem_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    r = subprocess.run(["make", "-C", str(ROOT / "oracle")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    _built = True


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    _build_once()
    yield


# Checkout of the reference project (read-only; only its shipped example
# meshes are read): DG_REFERENCE_DIR, else a sibling checkout named
# "reference" next to this repository.  Tests that need it skip without it.
REFERENCE = Path(os.environ["DG_REFERENCE_DIR"]) if "DG_REFERENCE_DIR" in os.environ else ROOT.parent / "reference"
