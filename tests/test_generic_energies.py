"""The nine further particle energies (types 6-14): the oracle's restatement checked on its
own (finite differences, known answers), the solver's per-vertex forward-mode blocks
(spg_gb300/csrc/generic.cuh) instantiated on the CPU against the oracle's full-element AD,
and, on a GB300, the device blocks and whole simulations against the oracle."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

GENERIC = (O.STVK_TET, O.SSNH, O.BW_MEMBRANE, O.CHOI_MEMBRANE, O.BW_BENDING, O.QUAD_BENDING, O.SPRING_CONT,
           O.SPRING_SQ_CONT, O.STATIC_LOAD)
LIB = os.path.join(os.path.dirname(__file__), "native", "libelements_host.so")
dp = C.POINTER(C.c_double)


def _variant_scenes():
    return {"stvk_tet_load": scenes.beam_tet_variant(O.STVK_TET, load=True), "ssnh": scenes.beam_tet_variant(O.SSNH),
            "bw": scenes.cloth_variant((O.BW_MEMBRANE, O.BW_BENDING)),
            "choi_quad": scenes.cloth_variant((O.CHOI_MEMBRANE, O.QUAD_BENDING)),
            "springs": scenes.spring_variant()}


def _cases(n_per_energy=12, seed=3):
    rng = np.random.default_rng(seed)
    for obj in _variant_scenes().values():
        scale = 0.03 * float(np.ptp(obj.x0, axis=0).max())
        for e in obj.energies:
            if e.type not in GENERIC:
                continue
            for i in rng.integers(0, e.n, size=min(n_per_energy, e.n)):
                X = obj.x[e.stencils[i]] + rng.normal(scale=scale, size=(e.stencils.shape[1], 3))
                for slot in range(e.stencils.shape[1]):
                    yield e.type, X, e.params[i], slot


def test_every_type_has_cases():
    assert {c[0] for c in _cases()} == set(GENERIC)


def test_oracle_gradient_matches_finite_differences():
    """Full-element and per-vertex AD agree, and the gradient is the energy's derivative
    (except Baraff-Witkin bending, whose norms are held constant by design)."""
    for etype, X, p, slot in _cases(4):
        g, H = O.element_block(etype, X, p, slot, O.FULL_AD)
        g2, H2 = O.element_block(etype, X, p, slot, O.VERTEX_AD)
        s = max(np.abs(g).max(), 1e-12)
        assert np.abs(g - g2).max() <= 1e-12 * s and np.abs(H - H2).max() <= 1e-12 * max(np.abs(H).max(), 1e-12)
        if etype == O.BW_BENDING:
            continue
        eps = 1e-6 * max(1.0, float(np.abs(X).max()))
        fd = np.zeros(3)
        for a in range(3):
            Xp, Xm = X.copy(), X.copy()
            Xp[slot, a] += eps
            Xm[slot, a] -= eps
            fd[a] = (O.element_energy(etype, Xp, p) - O.element_energy(etype, Xm, p)) / (2 * eps)
        assert np.abs(fd - g).max() <= 1e-6 * s + 1e-9, (etype, slot, fd, g)


def test_rest_state_is_stress_free():
    """At the rest positions every elastic energy has zero gradient (the load excepted)."""
    for obj in _variant_scenes().values():
        for e in obj.energies:
            if e.type not in GENERIC or e.type == O.STATIC_LOAD:
                continue
            for i in range(min(10, e.n)):
                X = obj.x0[e.stencils[i]]
                for slot in range(e.stencils.shape[1]):
                    g, _ = O.element_block(e.type, X, e.params[i], slot, O.FULL_AD)
                    assert np.abs(g).max() <= 1e-9 * max(1.0, np.abs(e.params[i]).max()), (e.type, slot)


@pytest.fixture(scope="module")
def host():
    if not os.path.exists(LIB):
        import __graft_entry__ as ge
        ge._build_test_helpers()
    return C.CDLL(LIB)


def _host_block(fn, etype, X, p, slot):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(p, dtype=np.float64)
    g, H = np.zeros(3), np.zeros(9)
    fn(etype, X.ctypes.data_as(dp), p.ctypes.data_as(dp), slot, g.ctypes.data_as(dp), H.ctypes.data_as(dp))
    return g, H.reshape(3, 3)


def test_fp64_forward_mode_blocks_equal_full_element_ad(host):
    for etype, X, p, slot in _cases():
        g, H = _host_block(host.host_block_f64, etype, X, p, slot)
        gr, Hr = O.element_block(etype, X, p, slot, O.FULL_AD)
        assert np.abs(g - gr).max() <= 1e-9 * max(np.abs(gr).max(), 1e-30), (etype, slot)
        assert np.abs(H - Hr).max() <= 1e-9 * max(np.abs(Hr).max(), 1e-30), (etype, slot)


def test_fp32_forward_mode_relative_error(host):
    eg, eh = [], []
    for etype, X, p, slot in _cases():
        X = X.astype(np.float32).astype(np.float64)
        p = p.astype(np.float32).astype(np.float64)
        g, H = _host_block(host.host_block_f32, etype, X, p, slot)
        gr, Hr = O.element_block(etype, X, p, slot, O.FULL_AD)
        eg.append(np.linalg.norm(g - gr) / max(np.linalg.norm(gr), 1e-30))
        if np.linalg.norm(Hr) > 0:
            eh.append(np.linalg.norm(H - Hr) / np.linalg.norm(Hr))
    assert np.median(eg) <= 1e-5 and np.median(eh) <= 1e-5


def test_oracle_steps_the_variant_scenes():
    for name, obj in _variant_scenes().items():
        s = O.Vbd(obj, 1 / 60, 1, 10, scenes.GRAVITY, O.VERTEX_AD)
        for _ in range(3):
            s.step()
        x, _ = s.state()
        assert np.all(np.isfinite(x)), name


# ----------------------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_device_blocks_match_oracle():
    N = pytest.importorskip("spg_gb300.native")
    by_type = {}
    for etype, X, p, slot in _cases():
        by_type.setdefault(etype, []).append((X, p, slot))
    for etype, rows in by_type.items():
        X = np.array([r[0] for r in rows]).astype(np.float32).astype(np.float64)
        P = np.array([r[1] for r in rows]).astype(np.float32).astype(np.float64)
        slots = np.array([r[2] for r in rows], np.int32)
        g, H = N.eval_vertex_blocks(etype, X, P, slots)
        rel = []
        for i in range(len(rows)):
            gr, Hr = O.element_block(etype, X[i], P[i], int(slots[i]), O.FULL_AD)
            rel.append(np.linalg.norm(g[i] - gr) / max(np.linalg.norm(gr), 1e-30))
            if np.linalg.norm(Hr) > 0:
                rel.append(np.linalg.norm(H[i] - Hr) / np.linalg.norm(Hr))
        assert np.median(rel) <= 1e-5 and np.quantile(rel, 0.95) <= 1e-3, (etype, np.median(rel))


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", [1, 2, 3])
@pytest.mark.parametrize("name", ["stvk_tet_load", "ssnh", "bw", "choi_quad", "springs"])
def test_positions_after_10_steps_match_oracle(name, kernel):
    N = pytest.importorskip("spg_gb300.native")
    obj = _variant_scenes()[name]
    kw = dict(dt=1 / 60, iterations=30, gravity=scenes.GRAVITY)
    gpu = N.VbdSolver([obj], kernel=kernel, **kw)
    assert gpu.launch()[0] == kernel
    ref = O.Vbd(obj, 1 / 60, 1, 30, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(10):
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = np.abs(xg - xr).max()
    print(f"{name}: max |dx| after 10 steps {err:.3g} m (extent {extent:.3g} m)")
    assert err <= 1e-4 * extent


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["stvk_tet_load", "bw", "choi_quad", "springs"])
def test_tile_kernels_run_these_energies_bit_exactly(name):
    """Energies 6-14 in the tile records (one 16-byte record per incidence, parameters in the
    generic table): the per-colour tile launches and the dataflow kernel run the same sweeps,
    bit for bit, with the same lanes and tile size."""
    N = pytest.importorskip("spg_gb300.native")
    obj = _variant_scenes()[name]
    kw = dict(dt=1 / 60, iterations=20, gravity=scenes.GRAVITY, lanes_per_vertex=4, tile_vertices=32)
    a = N.VbdSolver([obj], kernel=2, **kw)
    b = N.VbdSolver([obj], kernel=3, **kw)
    for _ in range(3):
        a.step()
        b.step()
    assert np.array_equal(a.state(0)[0], b.state(0)[0])


@pytest.mark.gpu
def test_xpbd_refuses_the_static_load():
    N = pytest.importorskip("spg_gb300.native")
    with pytest.raises(N.SpgxError, match="load"):
        N.XpbdSolver([scenes.spring_variant(load=True)], dt=1 / 60, substeps=2, gravity=scenes.GRAVITY)


def _xpbd_scenes():
    v = _variant_scenes()
    v["stvk_tet"] = scenes.beam_tet_variant(O.STVK_TET)
    del v["stvk_tet_load"]
    return v


def test_oracle_xpbd_steps_the_variant_scenes():
    for name, obj in _xpbd_scenes().items():
        s = O.Xpbd(obj, 1 / 60, 4, scenes.GRAVITY)
        for _ in range(3):
            s.step()
        x, _ = s.state()
        assert np.all(np.isfinite(x)), name


@pytest.mark.gpu
def test_device_constraints_match_oracle():
    N = pytest.importorskip("spg_gb300.native")
    by_type = {}
    for etype, X, p, slot in _cases():
        if etype != O.STATIC_LOAD and slot == 0:
            by_type.setdefault(etype, []).append((X, p))
    for etype, rows in by_type.items():
        X = np.array([r[0] for r in rows]).astype(np.float32).astype(np.float64)
        P = np.array([r[1] for r in rows]).astype(np.float32).astype(np.float64)
        c, g = N.eval_constraints(etype, X, P)
        for i in range(len(rows)):
            cr, gr = O.element_constraints(etype, X[i], P[i])
            assert np.abs(c[i] - cr).max() <= 1e-4 * max(1.0, np.abs(cr).max()), etype
            assert np.abs(g[i] - gr).max() <= 1e-4 * max(1.0, np.abs(gr).max()), etype


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["stvk_tet", "ssnh", "bw", "choi_quad", "springs"])
def test_xpbd_positions_match_oracle(name):
    N = pytest.importorskip("spg_gb300.native")
    obj = _xpbd_scenes()[name]
    gpu = N.XpbdSolver([obj], dt=1 / 60, substeps=8, gravity=scenes.GRAVITY)
    ref = O.Xpbd(obj, 1 / 60, 8, scenes.GRAVITY)
    for _ in range(10):
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = np.abs(xg - xr).max()
    print(f"XPBD {name}: max |dx| after 10 steps {err:.3g} m (extent {extent:.3g} m)")
    assert err <= 1e-4 * extent
