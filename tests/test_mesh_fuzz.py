"""Malformed .msh files fail with an error, never a crash: specific cases
(tags, group dimensions, quotes, counts, block dimensions) and a seeded
fuzz of truncated and byte-corrupted ASCII 4.1, 4.0 (parametric) and 2.2
and binary 4.1 and 2.2 files, run in a child process so that a crash fails the test instead of
ending the session."""
from __future__ import annotations

import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

import dgcuda as D

HERE = Path(__file__).resolve().parent


def _ascii(tmp_path):
    m = D.Mesh.box_tri(2, 2, order=2, side_names=("Reflecting", "Absorbing") * 2)
    p = tmp_path / "a.msh"
    m.write_msh(p)
    return p.read_text()


def _nodes_block(text):
    a = text.index("$Nodes\n")
    return a, text.index("$EndNodes")


@pytest.mark.parametrize("case", ["node_tag_zero", "duplicate_node", "element_tag_negative", "group_dim",
                                  "unterminated", "huge_count", "block_dim"])
def test_malformed_ascii_files_fail_cleanly(tmp_path, case):
    text = _ascii(tmp_path)
    lines = text.split("\n")
    if case == "node_tag_zero":
        a = lines.index("$Nodes")
        lines[a + 3] = "0"                      # first tag of the first block
    elif case == "duplicate_node":
        a = lines.index("$Nodes")
        lines[a + 4] = lines[a + 3]
    elif case == "element_tag_negative":
        a = lines.index("$EndElements")
        f = lines[a - 1].split()
        f[1] = "-3"
        lines[a - 1] = " ".join(f)
    elif case == "group_dim":
        a = lines.index("$PhysicalNames")
        f = lines[a + 2].split(None, 2)
        lines[a + 2] = "12 " + f[1] + " " + f[2]
    elif case == "unterminated":
        a = lines.index("$PhysicalNames")
        lines[a + 2] = lines[a + 2].rstrip('"')
        del lines[a + 3:lines.index("$EndPhysicalNames") + 1]
        lines = lines[:a + 3]
    elif case == "huge_count":
        a = lines.index("$Nodes")
        f = lines[a + 1].split()
        f[1] = "2000000000"
        lines[a + 1] = " ".join(f)
    elif case == "block_dim":
        # walk the blocks to the triangles' header and declare it on a curve
        at = lines.index("$Elements") + 1
        nblk = int(lines[at].split()[0])
        at += 1
        for _ in range(nblk):
            f = lines[at].split()
            if f[0] == "2":
                f[0] = "1"
                lines[at] = " ".join(f)
                break
            at += 1 + int(f[3])
        else:
            raise AssertionError("no triangle block")
    p = tmp_path / "bad.msh"
    p.write_text("\n".join(lines))
    with pytest.raises(RuntimeError):
        D.Precomp(D.Mesh.read_msh(p))


FUZZ = textwrap.dedent("""
    import os, random, sys
    sys.path.insert(0, {pkg!r}); sys.path.insert(0, {tests!r})
    import dgcuda as D
    from msh_binary import (parse_msh41, with_parametric_nodes, write_msh22_ascii, write_msh22_binary,
                            write_msh40_ascii, write_msh41_binary)
    d = {tmp!r}
    m = D.Mesh.box_tet(2, 1, 1, order=2, side_names=("Absorbing", "Reflecting") * 3)
    src = os.path.join(d, "a.msh"); m.write_msh(src)
    p = parse_msh41(src)
    b41 = os.path.join(d, "b41.msh"); write_msh41_binary(p, b41)
    b22 = os.path.join(d, "b22.msh"); write_msh22_binary(p, b22)
    a40 = os.path.join(d, "a40.msh"); write_msh40_ascii(with_parametric_nodes(p), a40)
    a22 = os.path.join(d, "a22.msh"); write_msh22_ascii(p, a22)
    rng = random.Random(2026)
    counts = [0, 0]
    for path in (src, b41, b22, a40, a22):
        data = open(path, "rb").read()
        cases = [data[:k] for k in range(0, len(data), max(1, len(data) // 60))]
        for _ in range(140):
            b = bytearray(data)
            for _ in range(rng.randint(1, 8)):
                b[rng.randrange(len(b))] = rng.randrange(256)
            cases.append(bytes(b))
        for blob in cases:
            f = os.path.join(d, "case.msh")
            open(f, "wb").write(blob)
            try:
                D.Precomp(D.Mesh.read_msh(f))
                counts[0] += 1
            except RuntimeError:
                counts[1] += 1
    print("loaded", counts[0], "rejected", counts[1])
""")


def test_fuzzed_files_never_crash(tmp_path):
    code = FUZZ.format(pkg=str(D.PKG), tests=str(HERE), tmp=str(tmp_path))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    assert "rejected" in r.stdout
