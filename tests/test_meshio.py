"""Mesh input (spg::io::loadObj / loadMsh) and the scene builders over loaded meshes.

The C++ readers run on the host and are checked against the pure-Python restatement in
``oracle/meshio_ref.py`` on generated files, and against the arrays the files were written
from. No GPU is needed."""
import os

import numpy as np
import pytest

from oracle import meshio_ref as R
from tests import meshfiles as MF

S = pytest.importorskip("spg_gb300.scenes")
N = pytest.importorskip("spg_gb300.native")


def _grid_faces(rows, cols):
    """The triangles of buildTriangleSquareMesh (alternating diagonals)."""
    F = []
    for r in range(1, rows):
        for c in range(1, cols):
            if (r + c) % 2 == 0:
                F += [[r * cols + c - 1, (r - 1) * cols + c - 1, (r - 1) * cols + c],
                      [r * cols + c - 1, (r - 1) * cols + c, r * cols + c]]
            else:
                F += [[(r - 1) * cols + c - 1, r * cols + c, r * cols + c - 1],
                      [(r - 1) * cols + c - 1, (r - 1) * cols + c, r * cols + c]]
    return np.array(F, np.int32)


def _same(a, b):
    assert np.array_equal(a[0], b[0]) and a[0].dtype == b[0].dtype
    assert np.array_equal(a[1], b[1])


# ----------------------------------------------------------------------------------- OBJ


def test_obj_triangles_and_float_positions(tmp_path):
    rng = np.random.default_rng(0)
    V = rng.normal(size=(40, 3)) * 3
    F = rng.integers(0, 40, size=(60, 3))
    F = F[(F[:, 0] != F[:, 1]) & (F[:, 1] != F[:, 2]) & (F[:, 0] != F[:, 2])]
    for style in ("v", "v/vt", "v//vn", "v/vt/vn"):
        p = str(tmp_path / f"m_{style.replace('/', '_')}.obj")
        MF.write_obj(p, V, F, header="# generated\nmtllib none.mtl", corner_style=style)
        got = S.load_obj(p)
        # positions are float values widened to double, as tinyobjloader's real_t = float gives
        assert np.array_equal(got[0], V.astype(np.float32).astype(np.float64))
        assert np.array_equal(got[1], F)
        _same(got, R.load_obj(p))


def test_obj_polygons_negative_indices_and_first_shape(tmp_path):
    text = "\r\n".join([
        "# quads, a pentagon, negative indices, vt/vn lines, two shapes",
        "o first",
        "v 0 0 0", "v 2 0 0", "v 2.1 1 0", "v 0 1 0",        # quad with |p0-p2| > |p1-p3|
        "vt 0 0", "vn 0 0 1",
        "f 1 2 3 4",
        "v 0 0 1", "v 1 0 1", "v 3 1 1", "v 0 1 1",          # quad with |p0-p2| > |p1-p3| reversed
        "f -1 -2 -3 -4",
        "v 0 0 2", "v 1 0 2", "v 1.5 0.5 2", "v 1 1 2", "v 0 1 2",
        "f 9/1/1 10/1/1 11/1/1 12/1/1 13/1/1",                # pentagon: fan from corner 0
        "f 1 2",                                              # degenerate: dropped
        "g second",
        "v 5 5 5",
        "f 1 2 14",                                           # second shape: not returned
        "",
    ])
    p = str(tmp_path / "poly.obj")
    with open(p, "w") as fh:
        fh.write(text)
    V, F = S.load_obj(p)
    assert V.shape == (14, 3)   # every vertex of the file
    d02 = np.sum((V[2] - V[0]) ** 2)
    d13 = np.sum((V[3] - V[1]) ** 2)
    assert d02 > d13
    expect = [[0, 1, 3], [1, 2, 3]]
    # second quad: corners (7, 6, 5, 4) (negative indices count back from vertex 8)
    q = [7, 6, 5, 4]
    e02 = np.sum((V[q[2]] - V[q[0]]) ** 2)
    e13 = np.sum((V[q[3]] - V[q[1]]) ** 2)
    expect += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]] if e02 < e13 else [[q[0], q[1], q[3]], [q[1], q[2], q[3]]]
    expect += [[8, 9, 10], [8, 10, 11], [8, 11, 12]]
    assert F.tolist() == expect
    _same((V, F), R.load_obj(p))


@pytest.mark.parametrize("body,msg", [
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", "face index 0"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n", "out of range"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf -4 1 2\n", "out of range"),
    ("v 0 0 0\nv 1 0 0\n", "no faces"),
    ("v 0 x 0\nf 1 1 1\n", "bad vertex"),
])
def test_obj_errors(tmp_path, body, msg):
    p = str(tmp_path / "bad.obj")
    with open(p, "w") as fh:
        fh.write(body)
    with pytest.raises(N.SpgxError, match=msg):
        S.load_obj(p)


def test_missing_file(tmp_path):
    with pytest.raises(N.SpgxError, match="cannot open"):
        S.load_obj(str(tmp_path / "nope.obj"))
    with pytest.raises(N.SpgxError, match="cannot open"):
        S.load_msh(str(tmp_path / "nope.msh"))


def test_obj_shell_scene_equals_spring_cloth_builder(tmp_path):
    """The spring cloth written to OBJ and read back (float positions) builds, through the mesh
    shell builder, the scene the grid builder makes from the same float positions."""
    n = 33
    ref = S.spring_cloth(n).objects[0]
    F = _grid_faces(n, n)
    V32 = ref.x0.astype(np.float32).astype(np.float64)
    p = str(tmp_path / "cloth.obj")
    MF.write_obj(p, ref.x0, F)
    V, F2 = S.load_obj(p)
    assert np.array_equal(V, V32) and np.array_equal(F2, F)
    w = 2.0 * (n - 1) / 512
    a = S.triangle_mesh(V, F2, mass=0.1 * w * w, spring_k=1e4, bending=1e-4, anchor_k=1e5,
                        anchors=np.arange(n)).objects[0]
    b = S.triangle_mesh(V32, F, mass=0.1 * w * w, spring_k=1e4, bending=1e-4, anchor_k=1e5,
                        anchors=np.arange(n)).objects[0]
    assert [e.type for e in a.energies] == [e.type for e in ref.energies]
    for ea, eb, er in zip(a.energies, b.energies, ref.energies):
        assert np.array_equal(ea.stencils, er.stencils)   # same topology as the grid builder
        assert np.array_equal(ea.params, eb.params)
    # with the double positions, the shell builder reproduces the grid builder bit for bit
    c = S.triangle_mesh(ref.x0, F, mass=0.1 * w * w, spring_k=1e4, bending=1e-4, anchor_k=1e5,
                        anchors=np.arange(n)).objects[0]
    assert np.array_equal(c.mass, ref.mass) and np.array_equal(c.x, ref.x)
    for ec, er in zip(c.energies, ref.energies):
        assert np.array_equal(ec.stencils, er.stencils) and np.array_equal(ec.params, er.params)


# ----------------------------------------------------------------------------------- MSH


def _beam(nx=6, ny=4, nz=3):
    o = S.tet_beam(nx, ny, nz).objects[0]
    return o, o.x0, next(e for e in o.energies if e.stencils.shape[1] == 4).stencils


@pytest.mark.parametrize("fmt", ["2.2", "4.1", "4.1-binary"])
def test_msh_round_trip(tmp_path, fmt):
    _, V, T = _beam()
    p = str(tmp_path / f"beam_{fmt}.msh")
    tri = T[:5, :3]
    if fmt == "2.2":
        MF.write_msh22(p, V, T, extra_elements=[(2, list(t)) for t in tri] + [(1, [0, 1])])
    else:
        MF.write_msh41(p, V, T, binary=fmt.endswith("binary"), node_blocks=3, tri_block=tri)
    got = S.load_msh(p)
    assert np.array_equal(got[0], V) and np.array_equal(got[1], T)
    _same(got, R.load_msh(p))


@pytest.mark.parametrize("binary", [False, True])
def test_msh_node_tags_map_to_file_positions(tmp_path, binary):
    _, V, T = _beam(4, 3, 3)
    rng = np.random.default_rng(3)
    tags = rng.permutation(np.arange(100, 100 + len(V)))
    p = str(tmp_path / "tags.msh")
    MF.write_msh41(p, V, T, binary=binary, node_tags=tags)
    got = S.load_msh(p)
    assert np.array_equal(got[0], V) and np.array_equal(got[1], T)
    _same(got, R.load_msh(p))


@pytest.mark.parametrize("edit,msg", [
    (lambda s: s.replace("4.1 0 8", "3.0 0 8"), "not supported"),
    (lambda s: s.replace("3 1 0 ", "3 1 1 ", 1), "parametric"),
    (lambda s: s.replace("$EndNodes", "$EndNodez"), "EndNodes"),
])
def test_msh_errors(tmp_path, edit, msg):
    _, V, T = _beam(3, 3, 3)
    p = str(tmp_path / "bad.msh")
    MF.write_msh41(p, V, T)
    with open(p) as fh:
        s = fh.read()
    with open(p, "w") as fh:
        fh.write(edit(s))
    with pytest.raises(N.SpgxError, match=msg):
        S.load_msh(p)


def test_msh_solid_scene_equals_beam_builder(tmp_path):
    """A bar written to MSH and read back builds, through the tet-mesh builder with the x-min
    face anchored, the same packed scene as the beam builder, bit for bit."""
    nx, ny, nz, cell = 9, 4, 4, 0.025
    ref = S.tet_beam(nx, ny, nz, cell=cell).objects[0]
    T = next(e for e in ref.energies if e.stencils.shape[1] == 4).stencils
    p = str(tmp_path / "bar.msh")
    MF.write_msh41(p, ref.x0, T, binary=True)
    V, T2 = S.load_msh(p)
    sx, sy, sz = cell * (nx - 1), cell * (ny - 1), cell * (nz - 1)
    o = S.tet_mesh(V, T2, mass=1000.0 * sx * sy * sz, young=1e6, poisson=0.45, anchor_k=1e4,
                   anchors=np.arange(ny * nz)).objects[0]
    assert np.array_equal(o.mass, ref.mass) and np.array_equal(o.x, ref.x) and np.array_equal(o.x0, ref.x0)
    assert [e.type for e in o.energies] == [e.type for e in ref.energies]
    for a, b in zip(o.energies, ref.energies):
        assert np.array_equal(a.stencils, b.stencils) and np.array_equal(a.params, b.params)


def test_mesh_builders_validate(tmp_path):
    _, V, T = _beam(3, 3, 3)
    with pytest.raises(N.SpgxError, match="anchor"):
        S.tet_mesh(V, T, anchors=[len(V)])
    with pytest.raises(N.SpgxError):
        S.tet_mesh(V, T[:, [1, 0, 2, 3]])   # inverted tets: the SNH precomputation refuses them
    with pytest.raises(N.SpgxError):
        S.triangle_mesh(V[:3], [[0, 1, 5]])  # face index out of range


def test_large_files_parse(tmp_path):
    """A 129x129 cloth OBJ and a 20x10x10 bar in binary MSH parse to the written arrays."""
    n = 129
    ref = S.spring_cloth(n).objects[0]
    F = _grid_faces(n, n)
    p = str(tmp_path / "big.obj")
    MF.write_obj(p, ref.x0, F)
    V, F2 = S.load_obj(p)
    assert np.array_equal(F2, F) and np.array_equal(V, ref.x0.astype(np.float32).astype(np.float64))
    _, Vb, Tb = _beam(20, 10, 10)
    q = str(tmp_path / "big.msh")
    MF.write_msh41(q, Vb, Tb, binary=True, node_blocks=4)
    Vq, Tq = S.load_msh(q)
    assert np.array_equal(Vq, Vb) and np.array_equal(Tq, Tb)
    assert os.path.getsize(q) > 0


# ----------------------------------------------------------------------------------- GPU


def _oracle_object(o):
    from oracle import pyoracle as O
    return O.SceneObject(o.x.copy(), o.mass.copy(), [O.Energy(e.type, e.stencils.copy(), e.params.copy())
                                                     for e in o.energies], None, o.x0.copy())


def _vbd_parity(obj, dt, iters, steps=10):
    from oracle import pyoracle as O
    g = (0.0, 0.0, -9.81)
    gpu = N.VbdSolver([obj], dt=dt, iterations=iters, gravity=g)
    ref = O.Vbd(_oracle_object(obj), dt, 1, iters, g, O.VERTEX_AD)
    for _ in range(steps):
        gpu.step()
        ref.step()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(gpu.state(0)[0] - ref.state()[0]).max())
    return err, extent


@pytest.mark.gpu
def test_vbd_on_a_curved_shell_read_from_obj(tmp_path):
    """A curved 25x25 quad sheet written as OBJ quads, triangulated by the reader, built into a
    spring/bending shell with one edge anchored: GPU VBD within 1e-4 x extent of the FP64
    oracle after 10 steps."""
    n = 25
    u, v = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    V = np.stack([u, v, 0.15 * np.sin(3 * u) * np.cos(2 * v)], axis=-1).reshape(-1, 3)
    quads = [[i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1] for i in range(n - 1) for j in range(n - 1)]
    p = str(tmp_path / "shell.obj")
    MF.write_obj(p, V, quads)
    Vr, F = S.load_obj(p)
    assert len(F) == 2 * len(quads)
    obj = S.triangle_mesh(Vr, F, mass=0.2, spring_k=5e3, bending=1e-3, anchor_k=1e5, anchors=np.arange(n)).objects[0]
    err, extent = _vbd_parity(obj, 1 / 120, 20)
    print(f"OBJ shell max position error {err:.3e} m (extent {extent:.3f} m)")
    assert err <= 1e-4 * extent


@pytest.mark.gpu
def test_vbd_on_a_solid_read_from_msh(tmp_path):
    """A bar written as binary MSH 4.1 and read back: GPU VBD within 1e-4 x extent of the FP64
    oracle after 10 steps, and bit-identical to the same bar from the beam builder."""
    ref = S.tet_beam(11, 4, 4).objects[0]
    T = next(e for e in ref.energies if e.stencils.shape[1] == 4).stencils
    p = str(tmp_path / "bar.msh")
    MF.write_msh41(p, ref.x0, T, binary=True)
    V, T2 = S.load_msh(p)
    cell = 0.025
    mass = 1000.0 * (cell * 10) * (cell * 3) * (cell * 3)
    obj = S.tet_mesh(V, T2, mass=mass, young=1e6, poisson=0.45, anchor_k=1e4, anchors=np.arange(16)).objects[0]
    err, extent = _vbd_parity(obj, 1 / 60, 50)
    print(f"MSH solid max position error {err:.3e} m (extent {extent:.3f} m)")
    assert err <= 1e-4 * extent
    a = N.VbdSolver([obj], dt=1 / 60, iterations=50, gravity=(0, 0, -9.81), kernel=1)
    b = N.VbdSolver([ref], dt=1 / 60, iterations=50, gravity=(0, 0, -9.81), kernel=1)
    for _ in range(3):
        a.step()
        b.step()
    assert np.array_equal(a.state(0)[0], b.state(0)[0])
