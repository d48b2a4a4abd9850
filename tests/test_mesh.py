"""Mesh layer: generators, .msh reading/writing, and the product's
reference-semantics precompute against the oracle's (independent code)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O
from conftest import REFERENCE

GOLDEN = Path(__file__).parent / "golden"


def compare_precompute(mesh, bcs=None):
    pre = D.Precomp(mesh, bcs)
    a = pre.arrays()
    orc = O.Oracle(mesh.raw(), 1e-4, 340.0, 1.225, bcs=mesh.bcs() if bcs is None else bcs)
    b = orc.mesh()
    for k in ("fc", "el_f_ids", "el_f_orientation", "f_node_tags", "f_bc", "f_nbr_el_ids", "f_n_to_el_n_ids"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    assert np.abs(a["f_normals"] - b["f_normals"][:, 0, :]).max() < 1e-12
    assert np.allclose(a["f_jacobian_dets"], b["f_jacobian_dets"][:, 0], rtol=1e-12)
    assert np.allclose(a["el_jacobian_dets"], b["el_jacobian_dets"][:, 0], rtol=1e-12)
    return pre, a


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_box_tri_precompute_matches_oracle(order):
    m = D.Mesh.box_tri(4, 3, (-1, -1), (1, 0.5), order=order,
                       side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    pre, a = compare_precompute(m)
    K = 4 * 3 * 2
    assert pre.num_el == K
    nb = int(a["f_is_boundary"].sum())
    assert nb == 2 * (4 + 3)
    assert pre.f_num == (3 * K + nb) // 2
    assert a["fc"] == 1


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_box_tet_precompute_matches_oracle(order):
    m = D.Mesh.box_tet(2, 2, 2, order=order, side_names=("Absorbing", "Reflecting") * 3)
    pre, a = compare_precompute(m)
    K = 8 * 6
    assert pre.num_el == K
    nb = int(a["f_is_boundary"].sum())
    assert nb == 6 * 4 * 2
    assert pre.f_num == (4 * K + nb) // 2
    assert a["fc"] == (1 if order == 1 else -1)


def test_obstacles_become_boundary_faces():
    m = D.Mesh.box_tet(3, 3, 3, order=1, side_names=("Absorbing",) * 6, removed=[13],
                       obstacle_name="Reflecting")
    pre, a = compare_precompute(m)
    assert pre.num_el == 26 * 6
    refl = (a["f_bc"] == 1) & (a["f_is_boundary"] == 1)
    assert refl.sum() == 6 * 2  # the removed cell's six faces, two triangles each


def test_mesh_write_read_roundtrip(tmp_path):
    m = D.Mesh.box_tet(2, 1, 1, order=3, side_names=("Absorbing", "Reflecting") * 3)
    path = tmp_path / "box.msh"
    m.write_msh(path)
    m2 = D.Mesh.read_msh(path)
    r1, r2 = m.raw(), m2.raw()
    assert np.array_equal(r1["el_nodes"], r2["el_nodes"])
    assert np.allclose(r1["xyz"], r2["xyz"], rtol=0, atol=0)
    assert r1["phys_name"] == r2["phys_name"]
    for g in range(len(r1["phys_name"])):
        a = r1["phys_nodes"][r1["phys_offsets"][g]:r1["phys_offsets"][g + 1]]
        b = r2["phys_nodes"][r2["phys_offsets"][g]:r2["phys_offsets"][g + 1]]
        assert np.array_equal(a, b)
    p1, p2 = D.Precomp(m).arrays(), D.Precomp(m2).arrays()
    for k in ("el_f_ids", "f_bc", "el_f_orientation"):
        assert np.array_equal(p1[k], p2[k])


def test_read_msh22(tmp_path):
    text = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
2
1 7 "Reflecting"
2 8 "Domain"
$EndPhysicalNames
$Nodes
4
1 0 0 0
2 1 0 0
3 1 1 0
4 0 1 0
$EndNodes
$Elements
6
1 1 2 7 1 1 2
2 1 2 7 1 2 3
3 1 2 7 1 3 4
4 1 2 7 1 4 1
5 2 2 8 1 1 2 3
6 2 2 8 1 1 3 4
$EndElements
"""
    p = tmp_path / "sq.msh"
    p.write_text(text)
    m = D.Mesh.read_msh(p)
    r = m.raw()
    assert r["dim"] == 2 and r["order"] == 1 and len(r["el_tags"]) == 2
    assert list(r["el_tags"]) == [5, 6]
    assert m.bcs() == [(7, True)]
    compare_precompute(m)


def test_bad_inputs_fail_loudly(tmp_path):
    with pytest.raises(D.DGError):
        D.Mesh.read_msh(tmp_path / "missing.msh")
    bad = tmp_path / "bad.msh"
    bad.write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(D.DGError):
        D.Mesh.read_msh(bad)
    with pytest.raises(D.DGError):
        D.Mesh.box_tri(0, 3, order=3)
    with pytest.raises(D.DGError):
        D.Mesh.box_tet(2, 2, 2, order=6)


def _ref_mesh_paths():
    names = ["doc/2d/square.msh", "doc/2d/disk.msh", "doc/2d/square_reflection.msh", "doc/2d/room.msh",
             "doc/3d/cube.msh", "doc/3d/sphere.msh"]
    return [REFERENCE / n for n in names]


@pytest.mark.parametrize("path", _ref_mesh_paths(), ids=lambda p: p.name)
def test_reference_meshes(path):
    """The reference's shipped gmsh 4.0 meshes: counts against the committed
    golden file, Euler characteristic, and product == oracle precompute."""
    if not path.exists():
        pytest.skip("reference checkout not present")
    golden = json.loads((GOLDEN / "reference_meshes.json").read_text())[path.name]
    m = D.Mesh.read_msh(path)
    r = m.raw()
    bcs = [(int(t), n.startswith("Reflecting")) for d, t, n in zip(r["phys_dim"], r["phys_tag"], r["phys_name"])
           if d == r["dim"] - 1]
    pre, a = compare_precompute(m, bcs)
    nb = int(a["f_is_boundary"].sum())
    got = {"dim": r["dim"], "order": r["order"], "num_el": pre.num_el, "f_num": pre.f_num, "boundary_faces": nb,
           "phys": sorted(set(r["phys_name"]))}
    assert got == {k: v for k, v in golden.items() if k != "holes"}
    # Euler characteristic: V - E + F = 1 - holes for a planar domain
    V = len(np.unique(r["el_nodes"][:, :r["dim"] + 1]))
    if r["dim"] == 2:
        E = pre.f_num
        assert V - E + pre.num_el == 1 - golden.get("holes", 0)
    # every interior face has two neighbours, every boundary face one
    nbr = a["f_nbr_el_ids"]
    assert np.all((nbr[:, 1] >= 0) == (a["f_is_boundary"] == 0))


def _same_mesh(m1, m2):
    r1, r2 = m1.raw(), m2.raw()
    assert np.array_equal(r1["el_nodes"], r2["el_nodes"])
    assert np.array_equal(r1["xyz"], r2["xyz"])
    assert r1["phys_name"] == r2["phys_name"]
    for g in range(len(r1["phys_name"])):
        a = r1["phys_nodes"][r1["phys_offsets"][g]:r1["phys_offsets"][g + 1]]
        b = r2["phys_nodes"][r2["phys_offsets"][g]:r2["phys_offsets"][g + 1]]
        assert np.array_equal(a, b)
    p1, p2 = D.Precomp(m1).arrays(), D.Precomp(m2).arrays()
    for k in ("el_f_ids", "f_bc", "el_f_orientation", "f_nbr_el_ids", "f_n_to_el_n_ids"):
        assert np.array_equal(p1[k], p2[k]), k


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 3), (3, 2), (3, 4)])
@pytest.mark.parametrize("fmt", ["41-le", "41-be", "41-le-size4", "22-le", "22-be"])
def test_binary_msh_reads_like_ascii(tmp_path, dim, order, fmt):
    from msh_binary import parse_msh41, write_msh22_binary, write_msh41_binary

    if dim == 2:
        m = D.Mesh.box_tri(3, 2, order=order, side_names=("Absorbing", "Reflecting") * 2)
    else:
        m = D.Mesh.box_tet(2, 1, 2, order=order, side_names=("Absorbing", "Reflecting") * 3)
    src = tmp_path / "ascii.msh"
    m.write_msh(src)
    parsed = parse_msh41(src)
    dst = tmp_path / "binary.msh"
    endian = ">" if fmt.endswith("be") else "<"
    if fmt.startswith("41"):
        write_msh41_binary(parsed, dst, endian=endian, dsize=4 if fmt.endswith("size4") else 8)
    else:
        write_msh22_binary(parsed, dst, endian=endian)
    _same_mesh(D.Mesh.read_msh(src), D.Mesh.read_msh(dst))


def test_binary_msh_errors(tmp_path):
    from msh_binary import parse_msh41, write_msh41_binary

    m = D.Mesh.box_tri(2, 2, order=2)
    src = tmp_path / "ascii.msh"
    m.write_msh(src)
    good = tmp_path / "good.msh"
    write_msh41_binary(parse_msh41(src), good)
    data = good.read_bytes()
    cases = {
        # binary MSH 4.0 uses other field types: refused rather than misread
        "v40.msh": (data.replace(b"4.1 1 8", b"4.0 1 8", 1), "4.0"),
        "marker.msh": (data.replace(b"4.1 1 8\n\x01\x00\x00\x00", b"4.1 1 8\n\x02\x00\x00\x00", 1), "endianness"),
        "cut.msh": (data[:data.index(b"$Nodes") + 40], "truncated|exceeds the file"),
        "size.msh": (data.replace(b"4.1 1 8", b"4.1 1 2", 1), "data size"),
    }
    for name, (blob, words) in cases.items():
        p = tmp_path / name
        p.write_bytes(blob)
        with pytest.raises(RuntimeError, match=words):
            D.Mesh.read_msh(p)


@pytest.mark.parametrize("fmt", ["40-ascii", "41-ascii", "41-binary"])
@pytest.mark.parametrize("parametric", [False, True])
def test_msh4_encodings_and_parametric_nodes(tmp_path, fmt, parametric):
    from msh_binary import (parse_msh41, with_parametric_nodes, write_msh40_ascii, write_msh41_ascii,
                            write_msh41_binary)

    m = D.Mesh.box_tet(2, 2, 1, order=3, side_names=("Absorbing", "Reflecting") * 3)
    src = tmp_path / "ascii.msh"
    m.write_msh(src)
    parsed = parse_msh41(src)
    if parametric:
        parsed = with_parametric_nodes(parsed)
    dst = tmp_path / "other.msh"
    {"40-ascii": write_msh40_ascii, "41-ascii": write_msh41_ascii, "41-binary": write_msh41_binary}[fmt](parsed, dst)
    _same_mesh(D.Mesh.read_msh(src), D.Mesh.read_msh(dst))


def test_msh22_ascii_encoding_reads_like_41(tmp_path):
    from msh_binary import parse_msh41, write_msh22_ascii

    m = D.Mesh.box_tet(2, 1, 2, order=2, side_names=("Absorbing", "Reflecting") * 3)
    src = tmp_path / "ascii.msh"
    m.write_msh(src)
    dst = tmp_path / "v22.msh"
    write_msh22_ascii(parse_msh41(src), dst)
    _same_mesh(D.Mesh.read_msh(src), D.Mesh.read_msh(dst))
