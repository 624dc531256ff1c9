"""Device-side setup for topology changes: the energies' preparePrecomputations and the VBD
incidence lists on the GPU, against the host classes (spg_gb300/host, through the CPU test
helper) and the host incidence builder."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

N = pytest.importorskip("spg_gb300.native")
LIB = os.path.join(os.path.dirname(__file__), "native", "libhost_packing.so")


@pytest.fixture(scope="module")
def host():
    if not os.path.exists(LIB):
        import __graft_entry__ as ge
        ge._build_test_helpers()
    return C.CDLL(LIB)


def _host_pack(host, etype, x0, stencils, args):
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    st = np.ascontiguousarray(stencils, dtype=np.int32)
    a = np.ascontiguousarray(args, dtype=np.float64)
    n = st.shape[0]
    out = np.zeros(n * O.PARAM_COUNT[etype])
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    rc = host.host_pack(etype, x0.shape[0], x0.ctypes.data_as(dp), n, st.ctypes.data_as(ip), a.ctypes.data_as(dp),
                        out.ctypes.data_as(dp))
    assert rc == 0
    return out.reshape(n, -1)


def _curved_sheet(n=12):
    """A curved sheet (non-zero rest bending angles): vertices and triangles."""
    u, v = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    V = np.stack([u, v, 0.2 * np.sin(3 * u) * np.cos(2 * v)], axis=-1).reshape(-1, 3)
    F = []
    for i in range(n - 1):
        for j in range(n - 1):
            a, b, c, d = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
            F += [[a, b, c], [a, c, d]]
    return V, np.array(F, np.int32)


def _cases():
    """(type, x0, stencils, host args, device material row or rows) for every energy type."""
    rng = np.random.default_rng(7)
    flat = scenes.cloth_cfg1(9)
    tris = next(e for e in flat.energies if e.type == O.STVK).stencils
    beam = scenes.beam_cfg2(6, 4, 4)
    tets = next(e for e in beam.energies if e.type == O.SNH).stencils
    xb = beam.x0 + rng.normal(scale=2e-3, size=beam.x0.shape)   # irregular tets, still positive
    from spg_gb300 import scenes as S
    V, F = _curved_sheet()
    shell = S.triangle_mesh(V, F).objects[0]
    bend = next(e for e in shell.energies if e.type == O.BENDING).stencils
    pairs = next(e for e in shell.energies if e.type == O.SPRING).stencils
    xa = np.arange(len(V), dtype=np.int32)[::3].reshape(-1, 1)
    anchor_rows = np.column_stack([V[xa[:, 0]], np.full(len(xa), 3e4)])
    return [
        (O.SPRING, V, pairs, [5e3], [0.0, 5e3]),
        (O.ANCHOR, V, xa, [3e4], anchor_rows),
        (O.BENDING, V, bend, [2e-3], [0.0, 2e-3]),
        (O.STVK, flat.x0, tris, [1e4, 0.3], [1e4, 0.3]),
        (O.SNH, xb, tets, [1e6, 0.45], [1e6, 0.45]),
        (O.STVK_TET, xb, tets, [1e6, 0.45], [1e6, 0.45]),
        (O.SSNH, xb, tets, [2e5, 0.3], [2e5, 0.3]),
        (O.BW_MEMBRANE, flat.x0, tris, [1e3, 2e3, 5e2], [1e3, 2e3, 5e2]),
        (O.CHOI_MEMBRANE, flat.x0, tris, [1e3, 2e3, 5e2], [1e3, 2e3, 5e2]),
        (O.BW_BENDING, V, bend, [1e-3], [0.0, 1e-3]),
        (O.QUAD_BENDING, V, bend, [1e-3], [0.0, 1e-3]),
        (O.SPRING_CONT, V, pairs, [5e3], [0.0, 5e3]),
        (O.SPRING_SQ_CONT, V, pairs, [5e3], [0.0, 5e3]),
        (O.STATIC_LOAD, V, xa, [2.0, 0.0, 3.0, 4.0], [2.0, 0.0, 3.0, 4.0]),
    ]


@pytest.mark.parametrize("case", range(14))
def test_host_precompute_abi_matches_host_classes(host, case):
    """The host ABI (the baseline of the device precompute) packs what the host classes pack."""
    etype, x0, st, args, mat = _cases()[case]
    assert np.array_equal(N.precompute_params(etype, st, x0, np.asarray(mat, np.float64), device=None),
                          _host_pack(host, etype, x0, st, args))


def test_material_counts():
    lib = N.lib()
    N.lib().spgx_material_count.restype = C.c_int32
    assert [lib.spgx_material_count(t) for t in range(16)] == [0, 2, 4, 2, 2, 2, 2, 2, 3, 3, 2, 2, 2, 2, 4, 0]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(14))
def test_device_precompute_matches_host_classes(host, case):
    """Every packed value equals the host classes' bit for bit, except the rest bending angles
    (atan2 on the device), which agree to a few ulp."""
    etype, x0, st, args, mat = _cases()[case]
    ref = _host_pack(host, etype, x0, st, args)
    assert np.array_equal(ref, N.precompute_params(etype, st, x0, np.asarray(mat, np.float64), device=None))
    got = N.precompute_params(etype, st, x0, np.asarray(mat, np.float64))
    assert got.shape == ref.shape
    if etype in (O.BENDING, O.BW_BENDING):
        assert np.array_equal(got[:, 1:], ref[:, 1:])
        assert np.max(np.abs(got[:, 0] - ref[:, 0])) <= 4 * np.finfo(float).eps * max(1.0, np.abs(ref[:, 0]).max())
        assert np.abs(ref[:, 0]).max() > 0.01   # the curved sheet has real rest angles
    else:
        assert np.array_equal(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("etype,x0,st,mat,msg", [
    (O.SNH, np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]]), [[1, 0, 2, 3]], [1e6, 0.45], "volume"),
    (O.STVK, np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.1]]), [[0, 1, 2]], [1e4, 0.3], "z=0"),
    (O.STVK, np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.0]]), [[0, 2, 1]], [1e4, 0.3], "area"),
    (O.BENDING, np.eye(4)[:, :3], [[0, 1, 2, 3]], [3.2, 1.0], "restTheta"),
    (O.QUAD_BENDING, np.eye(4)[:, :3], [[0, 1, 2, 3]], [0.1, 1.0], "quadratic"),
    (O.SPRING, np.zeros((2, 3)), [[0, 1]], [0.0, 1.0], "rest length"),
])
def test_device_precompute_rejects_what_the_reference_rejects(etype, x0, st, mat, msg):
    with pytest.raises(N.SpgxError, match=msg):
        N.precompute_params(etype, st, x0, np.asarray(mat, np.float64))


def _star(nv=50):
    """An object whose vertex 0 sits in hundreds of stencils (large incidence buckets)."""
    rng = np.random.default_rng(2)
    x = rng.normal(size=(nv, 3))
    pairs = np.column_stack([np.zeros(300, np.int32), rng.integers(1, nv, 300)]).astype(np.int32)
    anchors = rng.integers(0, 3, size=(400, 1)).astype(np.int32)
    return O.SceneObject(x, np.ones(nv), [O.Energy(O.ANCHOR, anchors, np.tile([0, 0, 0, 1.0, 1.0], (400, 1))),
                                          O.Energy(O.SPRING, pairs, np.tile([1.0, 1.0, 1.0], (300, 1))),
                                          O.Energy(O.ANCHOR, anchors[::-1].copy(), np.tile([0, 0, 0, 1.0, 1.0], (400, 1)))])


@pytest.mark.gpu
def test_device_incidences_bit_exact_with_host():
    objs = [scenes.cloth_cfg1(17), scenes.beam_cfg2(9, 5, 5), scenes.spring_cloth_cfg3(65),
            scenes.beam_tet_variant(O.STVK_TET, load=True),
            scenes.cloth_variant((O.BW_MEMBRANE, O.BW_BENDING)), _star()]
    for obj in objs:
        c1, e1 = N.incidences(obj)
        c2, e2 = N.incidences(obj, device=0)
        assert np.array_equal(c1, c2) and np.array_equal(e1, e2)
