"""Writers of OBJ and Gmsh MSH files for the mesh-input tests and the benchmark."""
from __future__ import annotations

import struct

import numpy as np


def _rows(fmt, arr):
    return "\n".join(fmt % tuple(r) for r in arr.tolist())


def write_obj(path, V, faces, header="", corner_style="v"):
    """Vertices with repr-exact reals; faces as 1-based corners in the given style
    ("v", "v/vt", "v//vn", "v/vt/vn")."""
    out = [header] if header else []
    out.append("\n".join("v %r %r %r" % tuple(map(float, v)) for v in np.asarray(V)))
    def corner(i):
        i = int(i) + 1
        return {"v": f"{i}", "v/vt": f"{i}/{i}", "v//vn": f"{i}//{i}", "v/vt/vn": f"{i}/{i}/{i}"}[corner_style]
    out.append("\n".join("f " + " ".join(corner(i) for i in f) for f in faces))
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def write_msh22(path, V, T, node_tags=None, extra_elements=()):
    """ASCII 2.2: nodes, then (type, nodes) extra elements, then the tets (element type 4)."""
    tags = np.arange(1, len(V) + 1) if node_tags is None else np.asarray(node_tags)
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(len(V))]
    lines += ["%d %r %r %r" % (t, *map(float, v)) for t, v in zip(tags, V)]
    lines += ["$EndNodes", "$Elements", str(len(extra_elements) + len(T))]
    eid = 1
    for etype, nodes in extra_elements:
        lines.append(" ".join(map(str, [eid, etype, 2, 0, 1] + [int(tags[n]) for n in nodes])))
        eid += 1
    for t in T:
        lines.append(" ".join(map(str, [eid, 4, 2, 0, 1] + [int(tags[n]) for n in t])))
        eid += 1
    lines.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_msh41(path, V, T, binary=False, node_blocks=2, tri_block=None, node_tags=None):
    """Format 4.1 with the nodes split over `node_blocks` entity blocks, an $Entities section
    (skipped by readers), an optional triangle block before the tets, ASCII or binary."""
    V = np.asarray(V, np.float64)
    T = np.asarray(T, np.int64)
    n = len(V)
    tags = np.arange(1, n + 1, dtype=np.int64) if node_tags is None else np.asarray(node_tags, np.int64)
    cuts = np.linspace(0, n, node_blocks + 1).astype(int)
    blocks = [(tri_block, 2)] if tri_block is not None else []
    blocks.append((T, 4))
    n_el = sum(len(b) for b, _ in blocks)
    with open(path, "wb") as fh:
        fh.write(b"$MeshFormat\n4.1 %d 8\n" % (1 if binary else 0))
        if binary:
            fh.write(struct.pack("<i", 1) + b"\n")
        fh.write(b"$EndMeshFormat\n$Entities\n0 0 0 1\n1 0 0 0 1 1 1 0 0\n$EndEntities\n$Nodes\n")
        if binary:
            fh.write(struct.pack("<4Q", node_blocks, n, int(tags.min()), int(tags.max())))
            for b in range(node_blocks):
                a, e = cuts[b], cuts[b + 1]
                fh.write(struct.pack("<iiiQ", 3, 1, 0, e - a))
                fh.write(tags[a:e].astype("<u8").tobytes())
                fh.write(V[a:e].astype("<f8").tobytes())
            fh.write(b"\n$EndNodes\n$Elements\n")
            fh.write(struct.pack("<4Q", len(blocks), n_el, 1, n_el))
            eid = 1
            for cells, etype in blocks:
                fh.write(struct.pack("<iiiQ", 3 if etype == 4 else 2, 1, etype, len(cells)))
                data = np.concatenate([np.arange(eid, eid + len(cells))[:, None], tags[np.asarray(cells)]], axis=1)
                fh.write(data.astype("<u8").tobytes())
                eid += len(cells)
            fh.write(b"\n$EndElements\n")
        else:
            out = ["%d %d %d %d" % (node_blocks, n, int(tags.min()), int(tags.max()))]
            for b in range(node_blocks):
                a, e = cuts[b], cuts[b + 1]
                out.append("3 1 0 %d" % (e - a))
                out.append(_rows("%d", tags[a:e, None]))
                out.append(_rows("%r %r %r", V[a:e]))
            out.append("$EndNodes\n$Elements")
            out.append("%d %d 1 %d" % (len(blocks), n_el, n_el))
            eid = 1
            for cells, etype in blocks:
                out.append("%d 1 %d %d" % (3 if etype == 4 else 2, etype, len(cells)))
                data = np.concatenate([np.arange(eid, eid + len(cells))[:, None], tags[np.asarray(cells)]], axis=1)
                out.append(_rows(" ".join(["%d"] * data.shape[1]), data))
                eid += len(cells)
            out.append("$EndElements\n")
            fh.write(("\n".join(s for s in out if s != "") + "").encode())
