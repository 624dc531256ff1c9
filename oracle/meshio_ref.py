"""Test infrastructure only: a pure-Python restatement of the mesh readers that the reference's
``spg::io::loadObj`` and ``spg::io::loadMsh`` (spg/source/geom/io/obj.cpp:9-35,
spg/source/geom/io/msh.cpp:10-40) delegate to: tinyobjloader and MshIO.

Parity unpinned: both libraries are empty git submodules in the reference checkout (no
commit recorded, so no pinned version). The rules restated here are their documented
behaviour on the parts loadObj/loadMsh consume:

- OBJ (tinyobjloader LoadObj defaults: triangulate on, real_t = float):
  - ``v`` lines give float positions (loadObj widens them to double);
  - ``f`` corners ``v``, ``v/vt``, ``v//vn``, ``v/vt/vn`` are 1-based, and a negative index
    counts back from the vertices read so far;
  - faces of fewer than 3 corners are dropped; quads are split along the shorter diagonal
    (float arithmetic); larger polygons are fanned from corner 0;
  - ``o``/``g`` close the current shape once it holds triangles, and only the first shape's
    triangles are returned.
- MSH (MshIO, formats 2.2 ASCII and 4.1 ASCII/binary): nodes in file order; tetrahedra
  (element type 4) in file order, with node tags mapped to file positions.

The oracle is the checker for the C++ readers on small files; nothing in the library imports it.
"""
from __future__ import annotations

import struct

import numpy as np

NODES_PER_ELEMENT = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 10: 9, 11: 10, 12: 27, 13: 18, 14: 14,
                     15: 1, 16: 8, 17: 20, 18: 15, 19: 13, 20: 9, 21: 10, 22: 12, 23: 15, 24: 15, 25: 21, 26: 4,
                     27: 5, 28: 6, 29: 20, 30: 35, 31: 56}


def load_obj(path):
    verts = []
    tris = []
    done = False
    with open(path, "rb") as f:
        text = f.read().decode("ascii")
    for raw in text.split("\n"):
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        parts = line.split()
        key = parts[0]
        if key == "v":
            xyz = [float(t) for t in parts[1:4]] + [0.0] * max(0, 3 - len(parts[1:4]))
            verts.append(np.float32(xyz))
        elif key == "f":
            nv = len(verts)
            idx = []
            for tok in parts[1:]:
                i = int(tok.split("/")[0])
                if i == 0:
                    raise ValueError("face index 0")
                i = i - 1 if i > 0 else nv + i
                if not 0 <= i < nv:
                    raise ValueError("face index out of range")
                idx.append(i)
            if done or len(idx) < 3:
                continue
            if len(idx) == 3:
                tris.append(idx)
            elif len(idx) == 4:
                p = [verts[i] for i in idx]
                d02 = p[2] - p[0]
                d13 = p[3] - p[1]
                s02 = np.float32(d02[0] * d02[0]) + np.float32(d02[1] * d02[1])
                s02 = np.float32(s02 + np.float32(d02[2] * d02[2]))
                s13 = np.float32(d13[0] * d13[0]) + np.float32(d13[1] * d13[1])
                s13 = np.float32(s13 + np.float32(d13[2] * d13[2]))
                if s02 < s13:
                    tris += [[idx[0], idx[1], idx[2]], [idx[0], idx[2], idx[3]]]
                else:
                    tris += [[idx[0], idx[1], idx[3]], [idx[1], idx[2], idx[3]]]
            else:
                tris += [[idx[0], idx[k], idx[k + 1]] for k in range(1, len(idx) - 1)]
        elif key in ("o", "g"):
            if tris:
                done = True
    if not tris:
        raise ValueError("no faces")
    V = np.array(verts, np.float32).astype(np.float64).reshape(-1, 3)
    return V, np.array(tris, np.int32).reshape(-1, 3)


def _sections_ascii(text):
    """Yields (name, list of tokens) per $Section of an ASCII file."""
    lines = text.split("\n")
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        i += 1
        if not ln:
            continue
        if not ln.startswith("$"):
            raise ValueError("expected a section")
        name = ln[1:]
        body = []
        while lines[i].strip() != "$End" + name:
            body += lines[i].split()
            i += 1
        i += 1
        yield name, body


def load_msh(path):
    with open(path, "rb") as f:
        data = f.read()
    head = data[: data.index(b"$EndMeshFormat")].decode("ascii", "replace").split()
    version, ftype = head[1], int(head[2])
    if ftype == 1:
        return _load_msh41_binary(data)
    nodes, tags, tets = [], [], []
    for name, tok in _sections_ascii(data.decode("ascii")):
        it = iter(tok)
        nxt = lambda: next(it)  # noqa: E731
        if name == "Nodes":
            if version == "2.2":
                for _ in range(int(nxt())):
                    tags.append(int(nxt()))
                    nodes.append([float(nxt()) for _ in range(3)])
            else:
                nb = int(nxt())
                [nxt() for _ in range(3)]
                for _ in range(nb):
                    nxt(), nxt()
                    if int(nxt()) != 0:
                        raise ValueError("parametric")
                    n = int(nxt())
                    tags += [int(nxt()) for _ in range(n)]
                    nodes += [[float(nxt()) for _ in range(3)] for _ in range(n)]
        elif name == "Elements":
            if version == "2.2":
                for _ in range(int(nxt())):
                    nxt()
                    et, nt = int(nxt()), int(nxt())
                    [nxt() for _ in range(nt)]
                    e = [int(nxt()) for _ in range(NODES_PER_ELEMENT[et])]
                    if et == 4:
                        tets.append(e)
            else:
                nb = int(nxt())
                [nxt() for _ in range(3)]
                for _ in range(nb):
                    nxt(), nxt()
                    et, n = int(nxt()), int(nxt())
                    for _ in range(n):
                        e = [int(nxt()) for _ in range(NODES_PER_ELEMENT[et] + 1)]
                        if et == 4:
                            tets.append(e[1:])
    return _finish(nodes, tags, tets)


def _load_msh41_binary(data):
    nodes, tags, tets = [], [], []
    p = data.index(b"$Nodes\n") + len(b"$Nodes\n")
    nb, _, _, _ = struct.unpack_from("<4Q", data, p)
    p += 32
    for _ in range(nb):
        _, _, par, n = struct.unpack_from("<iiiQ", data, p)
        p += 20
        if par != 0:
            raise ValueError("parametric")
        tags += list(struct.unpack_from(f"<{n}Q", data, p))
        p += 8 * n
        xyz = struct.unpack_from(f"<{3 * n}d", data, p)
        p += 24 * n
        nodes += [list(xyz[3 * j:3 * j + 3]) for j in range(n)]
    p = data.index(b"$Elements\n") + len(b"$Elements\n")
    nb, _, _, _ = struct.unpack_from("<4Q", data, p)
    p += 32
    for _ in range(nb):
        _, _, et, n = struct.unpack_from("<iiiQ", data, p)
        p += 20
        k = NODES_PER_ELEMENT[et] + 1
        vals = struct.unpack_from(f"<{k * n}Q", data, p)
        p += 8 * k * n
        if et == 4:
            tets += [list(vals[k * j + 1:k * j + 5]) for j in range(n)]
    return _finish(nodes, tags, tets)


def _finish(nodes, tags, tets):
    pos = {t: i for i, t in enumerate(tags)}
    T = np.array([[pos[t] for t in e] for e in tets], np.int32).reshape(-1, 4)
    return np.array(nodes, np.float64).reshape(-1, 3), T
