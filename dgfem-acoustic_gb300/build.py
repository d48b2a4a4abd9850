"""Builds the GB300 library (lib/libdgcuda.so) and the dgalerkin executable.

CUDA sources are compiled for sm_103a only; host C++ with g++.  Translation
units compile in parallel and are skipped when their object is newer than
every source and header of the package.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-O3", f"-I{INCLUDE}"]
CXX_FLAGS = ["-O3", "-fPIC", "-std=c++17", "-Wall", "-Wno-unused-function", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _newest_dep() -> float:
    files = list(CSRC.rglob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _sources() -> tuple[list[Path], list[Path]]:
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    return cu, cpp


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile everything; returns the path of libdgcuda.so."""
    LIB.mkdir(exist_ok=True)
    obj_dir = LIB / "obj"
    obj_dir.mkdir(exist_ok=True)
    newest = _newest_dep()
    nvcc = _nvcc()
    cu, cpp = _sources()
    tasks = []
    for src in cu:
        obj = obj_dir / (src.stem + ".cu.o")
        tasks.append((obj, [nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]))
    for src in cpp:
        obj = obj_dir / (src.stem + ".o")
        tasks.append((obj, ["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)]))
    todo = [(o, c) for o, c in tasks if not o.exists() or o.stat().st_mtime < newest]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_run, c) for _, c in todo]
            for f in futs:
                f.result()
    so = LIB / "libdgcuda.so"
    objs = [str(o) for o, _ in tasks if not o.name.startswith("dgalerkin_main")]
    if not so.exists() or so.stat().st_mtime < newest or todo:
        cuda_lib = _cuda_home() / "lib64"
        _run([nvcc, *ARCH, "-shared", "-o", str(so), *objs, f"-L{cuda_lib}", "-lcudart"])
    exe = LIB / "dgalerkin"
    main_obj = obj_dir / "dgalerkin_main.o"
    if main_obj.exists() and (not exe.exists() or exe.stat().st_mtime < so.stat().st_mtime or todo):
        _run(["g++", "-o", str(exe), str(main_obj), f"-L{LIB}", "-ldgcuda", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {so}")
    return so


if __name__ == "__main__":
    build(verbose=True)
