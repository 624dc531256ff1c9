"""Failure detection without a GPU fault: a bounded device-side wait that runs out is
reported as a status, and the solver keeps working (the VBD dataflow kernel's tile waits,
the XPBD persistent kernels' waits, the CG launch's grid barriers)."""
import time

import numpy as np
import pytest

from tests import scenes

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")
SPGX_ERR_TIMEOUT = 5


def test_dataflow_wait_runs_out_and_the_solver_recovers():
    obj = scenes.spring_cloth_cfg3(65)
    kw = dict(dt=1 / 120, iterations=20, gravity=scenes.GRAVITY, kernel=3)
    s = N.VbdSolver([obj], **kw)
    k, g, b = s.launch()
    assert k == 3
    twin = N.VbdSolver([obj], lanes_per_vertex=g, tile_vertices=b // g, **kw)
    assert twin.launch() == (k, g, b)
    s.step()
    twin.step()
    x0, v0 = s.state(0)
    # Both take the state through the FP64 host arrays (which drops delta bits below 2^-53 of
    # the position), so that their device representations match from here on.
    twin.set_state(0, *twin.state(0))
    s.test_stall_tile(3)   # a sweep counter nothing will ever reach
    t0 = time.time()
    with pytest.raises(N.SpgxError) as err:
        s.step()
    elapsed = time.time() - t0
    assert err.value.status == SPGX_ERR_TIMEOUT, err.value
    assert elapsed < 30, elapsed
    # The handle still works: from the state before the failed step it steps exactly like a
    # twin solver that never stalled.
    s.set_state(0, x0, v0)
    s.step()
    twin.step()
    assert np.array_equal(s.state(0)[0], twin.state(0)[0])
    print(f"stalled step returned after {elapsed:.2f} s")


def test_stall_hook_needs_the_dataflow_kernel():
    obj = scenes.spring_cloth_cfg3(9)
    s = N.VbdSolver([obj], dt=1 / 120, iterations=1, gravity=scenes.GRAVITY, kernel=1)
    with pytest.raises(N.SpgxError):
        s.test_stall_tile(0)


@pytest.mark.parametrize("kernel", [2, 3])
def test_xpbd_persistent_wait_runs_out_and_the_solver_recovers(kernel):
    """The XPBD persistent kernels' bounded waits: a chunk counter that no substep reaches
    (dataflow kernel) or a grid barrier counter that no barrier reaches (synchronised kernel)
    makes the step return a timeout status; restored to the state before that step, the handle
    steps exactly like a twin that never stalled."""
    obj = scenes.spring_cloth_cfg3(65)
    kw = dict(dt=1 / 120, substeps=10, gravity=scenes.GRAVITY, kernel=kernel)
    s = N.XpbdSolver([obj], **kw)
    twin = N.XpbdSolver([obj], **kw)
    s.step()
    twin.step()
    x0, v0 = s.state(0)
    twin.set_state(0, *twin.state(0))
    s.test_stall()
    t0 = time.time()
    with pytest.raises(N.SpgxError) as err:
        s.step()
    elapsed = time.time() - t0
    assert err.value.status == SPGX_ERR_TIMEOUT, err.value
    assert elapsed < 30, elapsed
    s.set_state(0, x0, v0)
    s.step()
    twin.step()
    assert np.array_equal(s.state(0)[0], twin.state(0)[0])
    print(f"stalled XPBD step returned after {elapsed:.2f} s")


def test_cg_barrier_wait_runs_out_and_the_solver_recovers():
    """The implicit solvers' CG launch: a grid barrier counter that no barrier completes makes
    every bounded wait run out; the step returns a timeout status, and restored to the state
    before that step the handle steps like a twin that never stalled (to 1e-9 m: the FP64
    assembly adds with atomics in no fixed order, and the CG amplifies those last-bit
    differences to about 1e-12 m)."""
    obj = scenes.truss_variant()
    kw = dict(dt=1 / 60, substeps=1, gravity=scenes.GRAVITY)
    s = N.ImplicitSolver([obj], **kw)
    twin = N.ImplicitSolver([obj], **kw)
    s.step()
    twin.step()
    x0, v0 = s.state(0)
    s.test_stall()
    t0 = time.time()
    with pytest.raises(N.SpgxError) as err:
        s.step()
    elapsed = time.time() - t0
    assert err.value.status == SPGX_ERR_TIMEOUT, err.value
    assert elapsed < 30, elapsed
    s.set_state(0, x0, v0)
    s.step()
    twin.step()
    assert np.abs(s.state(0)[0] - twin.state(0)[0]).max() <= 1e-9
    print(f"stalled CG step returned after {elapsed:.2f} s")
