"""Test helper: re-encodes an ASCII MSH 4.1 file (one element or node per
line, as the library's writer emits) as a binary MSH 4.1 or MSH 2.2 file,
following gmsh's published format descriptions independently of the
library's reader: in MSH 4.1 binary, counts and tags are size_t (data-size
bytes), entity tags, dimensions, types and physical tags int32, coordinates
float64; MSH 2.2 binary gives nodes as (int32 tag, 3 float64) and elements
in runs headed by (type, run length, tag count), each element (int32 tag,
int32 tags, int32 nodes).  The line after "file-type data-size" holds the
int32 1 in the file's byte order."""
from __future__ import annotations

import struct
from pathlib import Path


def parse_msh41(path: str | Path) -> dict:
    text = Path(path).read_text()

    def body(name: str) -> list[str]:
        a = text.index("$" + name + "\n") + len(name) + 2
        b = text.index("$End" + name)
        return text[a:b].strip("\n").split("\n")

    phys = []
    if "$PhysicalNames" in text:
        for ln in body("PhysicalNames")[1:]:
            d, tag, name = ln.split(None, 2)
            phys.append((int(d), int(tag), name.strip().strip('"')))
    tok = iter(" ".join(body("Entities")).split())
    counts = [int(next(tok)) for _ in range(4)]
    ents = []
    for d in range(4):
        for _ in range(counts[d]):
            tag = int(next(tok))
            box = [float(next(tok)) for _ in range(3 if d == 0 else 6)]
            ph = [int(next(tok)) for _ in range(int(next(tok)))]
            bnd = [int(next(tok)) for _ in range(int(next(tok)))] if d > 0 else []
            ents.append((d, tag, box, ph, bnd))
    lines = body("Nodes")
    nblk = int(lines[0].split()[0])
    at, nblocks = 1, []
    for _ in range(nblk):
        ed, et, par, n = (int(v) for v in lines[at].split())
        tags = [int(v) for v in lines[at + 1:at + 1 + n]]
        xyz = [[float(v) for v in ln.split()] for ln in lines[at + 1 + n:at + 1 + 2 * n]]
        nblocks.append((ed, et, par, tags, xyz))
        at += 1 + 2 * n
    lines = body("Elements")
    nblk = int(lines[0].split()[0])
    at, eblocks = 1, []
    for _ in range(nblk):
        ed, et, typ, n = (int(v) for v in lines[at].split())
        els = [[int(v) for v in ln.split()] for ln in lines[at + 1:at + 1 + n]]
        eblocks.append((ed, et, typ, els))
        at += 1 + n
    return {"phys": phys, "counts": counts, "ents": ents, "nodes": nblocks, "elements": eblocks}


def _phys_section(m: dict) -> bytes:
    if not m["phys"]:
        return b""
    out = b"$PhysicalNames\n%d\n" % len(m["phys"])
    for d, tag, name in m["phys"]:
        out += b'%d %d "%s"\n' % (d, tag, name.encode())
    return out + b"$EndPhysicalNames\n"


def write_msh41_binary(m: dict, path: str | Path, endian: str = "<", dsize: int = 8) -> None:
    S = "Q" if dsize == 8 else "I"

    def p(fmt, *v):
        return struct.pack(endian + fmt, *v)

    out = b"$MeshFormat\n4.1 1 %d\n" % dsize + p("i", 1) + b"\n$EndMeshFormat\n"
    out += _phys_section(m)
    out += b"$Entities\n" + p("4" + S, *m["counts"])
    for d, tag, box, ph, bnd in m["ents"]:
        out += p("i", tag) + p("%dd" % len(box), *box) + p(S, len(ph)) + p("%di" % len(ph), *ph)
        if d > 0:
            out += p(S, len(bnd)) + p("%di" % len(bnd), *bnd)
    out += b"\n$EndEntities\n"
    tags = [t for b in m["nodes"] for t in b[3]]
    out += b"$Nodes\n" + p("4" + S, len(m["nodes"]), len(tags), min(tags), max(tags))
    for ed, et, par, tg, xyz in m["nodes"]:
        out += p("3i", ed, et, par) + p(S, len(tg)) + p("%d%s" % (len(tg), S), *tg)
        flat = [c for x in xyz for c in x]  # x y z and any parametric coordinates
        out += p("%dd" % len(flat), *flat)
    out += b"\n$EndNodes\n"
    etags = [e[0] for b in m["elements"] for e in b[3]]
    out += b"$Elements\n" + p("4" + S, len(m["elements"]), len(etags), min(etags), max(etags))
    for ed, et, typ, els in m["elements"]:
        out += p("3i", ed, et, typ) + p(S, len(els))
        for e in els:
            out += p("%d%s" % (len(e), S), *e)
    out += b"\n$EndElements\n"
    Path(path).write_bytes(out)


def write_msh22_binary(m: dict, path: str | Path, endian: str = "<") -> None:
    def p(fmt, *v):
        return struct.pack(endian + fmt, *v)

    ent_phys = {(d, tag): (ph[0] if ph else 0) for d, tag, _, ph, _ in m["ents"]}
    out = b"$MeshFormat\n2.2 1 8\n" + p("i", 1) + b"\n$EndMeshFormat\n"
    out += _phys_section(m)
    nodes = [(t, x) for b in m["nodes"] for t, x in zip(b[3], b[4])]
    out += b"$Nodes\n%d\n" % len(nodes)
    for t, x in nodes:
        out += p("i3d", t, *x)
    out += b"\n$EndNodes\n"
    ne = sum(len(b[3]) for b in m["elements"])
    out += b"$Elements\n%d\n" % ne
    for ed, et, typ, els in m["elements"]:
        out += p("3i", typ, len(els), 2)
        for e in els:
            out += p("3i", e[0], ent_phys[(ed, et)], et) + p("%di" % (len(e) - 1), *e[1:])
    out += b"\n$EndElements\n"
    Path(path).write_bytes(out)


def _fmt(v) -> str:
    return repr(float(v))


def write_msh41_ascii(m: dict, path: str | Path) -> None:
    out = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat"]
    txt = _phys_section(m).decode()
    if txt:
        out += txt.strip("\n").split("\n")
    out += ["$Entities", " ".join(map(str, m["counts"]))]
    for d, tag, box, ph, bnd in m["ents"]:
        row = [str(tag)] + [_fmt(v) for v in box] + [str(len(ph))] + [str(v) for v in ph]
        if d > 0:
            row += [str(len(bnd))] + [str(v) for v in bnd]
        out.append(" ".join(row))
    out.append("$EndEntities")
    tags = [t for b in m["nodes"] for t in b[3]]
    out += ["$Nodes", f"{len(m['nodes'])} {len(tags)} {min(tags)} {max(tags)}"]
    for ed, et, par, tg, xyz in m["nodes"]:
        out.append(f"{ed} {et} {par} {len(tg)}")
        out += [str(t) for t in tg]
        out += [" ".join(_fmt(c) for c in x) for x in xyz]
    out.append("$EndNodes")
    etags = [e[0] for b in m["elements"] for e in b[3]]
    out += ["$Elements", f"{len(m['elements'])} {len(etags)} {min(etags)} {max(etags)}"]
    for ed, et, typ, els in m["elements"]:
        out.append(f"{ed} {et} {typ} {len(els)}")
        out += [" ".join(map(str, e)) for e in els]
    out.append("$EndElements")
    Path(path).write_text("\n".join(out) + "\n")


def write_msh40_ascii(m: dict, path: str | Path) -> None:
    """MSH 4.0: points carry a 6-value box, block headers give the entity tag
    before its dimension, nodes are "tag x y z [params]" lines, and the
    section headers have no tag ranges."""
    out = ["$MeshFormat", "4 0 8", "$EndMeshFormat"]
    txt = _phys_section(m).decode()
    if txt:
        out += txt.strip("\n").split("\n")
    out += ["$Entities", " ".join(map(str, m["counts"]))]
    for d, tag, box, ph, bnd in m["ents"]:
        b6 = box if d > 0 else box + box
        row = [str(tag)] + [_fmt(v) for v in b6] + [str(len(ph))] + [str(v) for v in ph]
        if d > 0:
            row += [str(len(bnd))] + [str(v) for v in bnd]
        out.append(" ".join(row))
    out.append("$EndEntities")
    nn = sum(len(b[3]) for b in m["nodes"])
    out += ["$Nodes", f"{len(m['nodes'])} {nn}"]
    for ed, et, par, tg, xyz in m["nodes"]:
        out.append(f"{et} {ed} {par} {len(tg)}")
        out += [f"{t} " + " ".join(_fmt(c) for c in x) for t, x in zip(tg, xyz)]
    out.append("$EndNodes")
    ne = sum(len(b[3]) for b in m["elements"])
    out += ["$Elements", f"{len(m['elements'])} {ne}"]
    for ed, et, typ, els in m["elements"]:
        out.append(f"{et} {ed} {typ} {len(els)}")
        out += [" ".join(map(str, e)) for e in els]
    out.append("$EndElements")
    Path(path).write_text("\n".join(out) + "\n")


def with_parametric_nodes(m: dict) -> dict:
    """The same mesh with every node block marked parametric: each node gains
    entityDim parametric coordinates after x y z."""
    m = dict(m)
    m["nodes"] = [(ed, et, 1, tg, [list(x) + [0.125 * (k + 1) for k in range(ed)] for x in xyz])
                  for ed, et, par, tg, xyz in m["nodes"]]
    return m


def write_msh22_ascii(m: dict, path: str | Path) -> None:
    """MSH 2.2 ASCII: "tag x y z" node lines and "tag type 2 physical
    elementary nodes..." element lines."""
    ent_phys = {(d, tag): (ph[0] if ph else 0) for d, tag, _, ph, _ in m["ents"]}
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat"]
    txt = _phys_section(m).decode()
    if txt:
        out += txt.strip("\n").split("\n")
    nodes = [(t, x) for b in m["nodes"] for t, x in zip(b[3], b[4])]
    out += ["$Nodes", str(len(nodes))] + [f"{t} " + " ".join(_fmt(c) for c in x[:3]) for t, x in nodes]
    out.append("$EndNodes")
    els = [(e, typ, ent_phys[(ed, et)], et) for ed, et, typ, es in m["elements"] for e in es]
    out += ["$Elements", str(len(els))]
    out += [f"{e[0]} {typ} 2 {ph} {et} " + " ".join(map(str, e[1:])) for e, typ, ph, et in els]
    out.append("$EndElements")
    Path(path).write_text("\n".join(out) + "\n")
