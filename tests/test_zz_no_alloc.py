"""The allocation-free element evaluation (spgx_eval_vertex_blocks_noalloc) against the
allocating entry point, through the C ABI. It serves callers that cannot allocate device
memory (their device memory belongs to another allocator, or allocation is not allowed after
start-up); its device staging is a fixed array inside the library, so it accepts at most
4096 incidences per call and two calls in a row reuse the same array."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")


def _scene_with(etype):
    """A scene object that holds energy type `etype` (the benchmark scenes for types 1-5, the
    test variants of the bar, cloth and spring cloth for types 6-14)."""
    from oracle import pyoracle as O
    from tests import scenes as T
    if etype in (O.BENDING, O.STVK):
        return T.cloth_cfg1(9)
    if etype == O.SNH:
        return T.beam_cfg2(5, 3, 3)
    if etype in (O.SPRING, O.ANCHOR):
        return T.spring_cloth_cfg3(17)
    if etype in (O.STVK_TET, O.SSNH):
        return T.beam_tet_variant(etype, 5, 3, 3)
    if etype == O.STATIC_LOAD:
        return T.beam_tet_variant(O.STVK_TET, 5, 3, 3, load=True)
    if etype in (O.BW_MEMBRANE, O.BW_BENDING):
        return T.cloth_variant((O.BW_MEMBRANE, O.BW_BENDING), 9)
    if etype in (O.CHOI_MEMBRANE, O.QUAD_BENDING):
        return T.cloth_variant((O.CHOI_MEMBRANE, O.QUAD_BENDING), 9)
    return T.spring_variant(9)


def _inputs(etype, n, seed):
    """Random incidences near the scene's own element shapes, with their energy parameters."""
    rng = np.random.default_rng(seed)
    obj = _scene_with(etype)
    e = next(e for e in obj.energies if e.type == etype)
    idx = rng.integers(0, e.n, size=n)
    X = obj.x[e.stencils[idx]] + rng.normal(scale=1e-3, size=(n, e.stencils.shape[1], 3))
    slots = rng.integers(0, e.stencils.shape[1], size=n)
    return X.reshape(n, -1), e.params[idx], slots


def _types():
    return [t for t in range(1, 15) if N.lib().spgx_stencil_size(t) > 0]


@pytest.mark.parametrize("etype", list(range(1, 15)))
def test_noalloc_matches_allocating_entry_point(etype):
    """Two calls in a row per energy type (the second reuses the array the first filled); the
    membrane StVK type, which has the most parameters per stencil (22), fills the whole array."""
    assert etype in _types()
    sizes = [(1000, 1), (4096, 2)] if etype == N.STVK else [(700, 1), (1500, 2)]
    for call, (n, seed) in enumerate(sizes):
        X, P, slots = _inputs(etype, n, seed + 10 * etype)
        g_ref, H_ref = N.eval_vertex_blocks(etype, X, P, slots)
        g, H = N.eval_vertex_blocks_noalloc(etype, X, P, slots)
        np.testing.assert_allclose(g, g_ref, rtol=1e-6, atol=0, err_msg=f"type {etype}, call {call}")
        np.testing.assert_allclose(H, H_ref, rtol=1e-6, atol=0, err_msg=f"type {etype}, call {call}")


def test_noalloc_rejects_more_than_capacity():
    X, P, slots = _inputs(N.SPRING, 4097, 5)
    with pytest.raises(N.SpgxError, match="capacity"):
        N.eval_vertex_blocks_noalloc(N.SPRING, X, P, slots)
