"""The allocation-free element evaluation (spgx_eval_vertex_blocks_noalloc) against the
allocating entry point, through the C ABI. It serves callers that cannot allocate device
memory (their device memory belongs to another allocator, or allocation is not allowed after
start-up); its device staging is a fixed array inside the library, so it accepts at most
4096 incidences per call and two calls in a row reuse the same array."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")


def _inputs(etype, n, seed):
    """Random incidences near the scenes' own element shapes, with their energy parameters."""
    from spg_gb300 import scenes as S
    rng = np.random.default_rng(seed)
    obj = (S.cloth(9).objects[0] if etype in (N.BENDING, N.STVK) else
           S.tet_beam(5, 3, 3).objects[0] if etype == N.SNH else S.spring_cloth(17).objects[0])
    e = next(e for e in obj.energies if e.type == etype)
    idx = rng.integers(0, e.n, size=n)
    X = obj.x[e.stencils[idx]] + rng.normal(scale=1e-3, size=(n, e.stencils.shape[1], 3))
    slots = rng.integers(0, e.stencils.shape[1], size=n)
    return X.reshape(n, -1), e.params[idx], slots


@pytest.mark.parametrize("etype", [N.SPRING, N.BENDING, N.STVK, N.SNH])
def test_noalloc_matches_allocating_entry_point(etype):
    for call, (n, seed) in enumerate([(1000, 1), (4096, 2)]):
        X, P, slots = _inputs(etype, n, seed + 10 * etype)
        g_ref, H_ref = N.eval_vertex_blocks(etype, X, P, slots)
        g, H = N.eval_vertex_blocks_noalloc(etype, X, P, slots)
        np.testing.assert_allclose(g, g_ref, rtol=1e-6, atol=0, err_msg=f"call {call}")
        np.testing.assert_allclose(H, H_ref, rtol=1e-6, atol=0, err_msg=f"call {call}")


def test_noalloc_rejects_more_than_capacity():
    X, P, slots = _inputs(N.SPRING, 4097, 5)
    with pytest.raises(N.SpgxError, match="capacity"):
        N.eval_vertex_blocks_noalloc(N.SPRING, X, P, slots)
