"""Interactive picking without a rebuild: dynamic anchors in the VBD solver against the FP64
oracle with the picking SpringAnchorEnergy appended, and the C++ GpuVBD drop-in driven
through the reference application's pick / drag / release sequence
(apps/solverCompare.cpp:717-726, 1496-1524)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")
GRAVITY = (0.0, 0.0, -9.81)
PICK_K = 1e4   # the application's particle picking stiffness (solverCompare.cpp:722)


def _with_anchor(obj, vertex, target, k):
    o = obj.copy()
    o.energies.append(O.Energy(O.ANCHOR, np.array([[vertex]], np.int32), np.array([[*target, k, 1.0 / k]])))
    return o


def _path(x0, steps):
    return np.array([x0 + np.array([0.004 * s, 0.0, 0.006 * s]) for s in range(steps)])


@pytest.mark.parametrize("scene", ["cloth", "beam"])
@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_pick_matches_oracle_with_appended_anchor(kernel, scene):
    """A pick on the free corner of the hanging cloth, or on the free end of the SNH bar: 10
    steps within 1e-4 x extent of the oracle with the anchor appended. (Both scenes are well
    conditioned: a 1e-9 m perturbation of the oracle's start stays below 1e-9 m; a pull of
    several centimetres on the cloth's corner is not, in the oracle itself.)"""
    if scene == "cloth":
        obj, dt, iters, d = scenes.spring_cloth_cfg3(33), 1 / 120, 20, np.array([0.01, 0.0, 0.01])
    else:
        obj, dt, iters, d = scenes.beam_cfg2(11, 4, 4), 1 / 60, 50, np.array([0.0, 0.0, 0.02])
    v = obj.nv - 1
    target = obj.x[v] + d
    gpu = N.VbdSolver([obj], dt=dt, iterations=iters, gravity=GRAVITY, kernel=kernel)
    gpu.set_picks([(0, v, target, PICK_K)])
    ref = O.Vbd(_with_anchor(obj, v, target, PICK_K), dt, 1, iters, GRAVITY, O.VERTEX_AD)
    free = O.Vbd(obj, dt, 1, iters, GRAVITY, O.VERTEX_AD)
    for _ in range(10):
        gpu.step()
        ref.step()
        free.step()
    xg, xr = gpu.state(0)[0], ref.state()[0]
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    print(f"pick on the {scene} (kernel {kernel}) max position error {err:.3e} m (extent {extent:.3f} m)")
    assert err <= 1e-4 * extent
    assert np.abs(xg - free.state()[0]).max() > 100 * err   # the pick changed the motion


def test_pick_drag_release_sequence_matches_oracle():
    """Pick at step 2, drag every step, release at step 7: each step against an oracle solver
    holding the energies of that moment, started from the previous step's oracle state."""
    obj = scenes.spring_cloth_cfg3(33)
    v, steps, start, end = obj.nv // 2 + 3, 10, 2, 7
    path = _path(obj.x[v], steps)
    gpu = N.VbdSolver([obj], dt=1 / 120, iterations=20, gravity=GRAVITY, kernel=1)
    x, vel = obj.x.copy(), np.zeros_like(obj.x)
    anchor = None
    for s in range(steps):
        if s == start:
            anchor = x[v].copy()
        if anchor is not None and s > start:
            anchor = path[s]
        if s == end:
            anchor = None
        gpu.set_picks([] if anchor is None else [(0, v, anchor, PICK_K)])
        o = obj if anchor is None else _with_anchor(obj, v, anchor, PICK_K)
        ref = O.Vbd(o, 1 / 120, 1, 20, GRAVITY, O.VERTEX_AD)
        ref.set_state(x, vel)
        ref.step()
        x, vel = ref.state()
        gpu.step()
    err = float(np.abs(gpu.state(0)[0] - x).max())
    print(f"pick sequence max position error {err:.3e} m")
    assert err <= 1e-4 * float(np.ptp(obj.x0, axis=0).max())


def test_residual_includes_the_pick():
    """The solver's residual norm counts the pick's force k (x - a): with picks at a = x +- d,
    (r+^2 + r-^2 - 2 r0^2) / 2 = k^2 |d|^2 whatever the other forces on the vertex."""
    obj = scenes.spring_cloth_cfg3(17)
    s = N.VbdSolver([obj], dt=1 / 120, iterations=0, gravity=GRAVITY)
    s.step()
    r0 = s.residual()
    v = obj.nv - 1
    x = s.state(0)[0][v]
    d = np.array([0.0, 0.0, 1.0])
    s.set_picks([(0, v, x + d, PICK_K)])
    rp = s.residual()
    s.set_picks([(0, v, x - d, PICK_K)])
    rm = s.residual()
    k_d = np.sqrt((rp ** 2 + rm ** 2 - 2 * r0 ** 2) / 2)
    assert abs(k_d - PICK_K) <= 1e-2 * PICK_K, (r0, rp, rm)


def test_pick_validation():
    obj = scenes.spring_cloth_cfg3(9)
    s = N.VbdSolver([obj], dt=1 / 120, iterations=1, gravity=GRAVITY)
    with pytest.raises(N.SpgxError, match="names no vertex"):
        s.set_picks([(0, obj.nv, (0, 0, 0), 1.0)])
    with pytest.raises(N.SpgxError, match="SPGX_MAX_PICKS"):
        s.set_picks([(0, 0, (0, 0, 0), 1.0)] * 17)


def _driver():
    lib = os.path.join(os.path.dirname(__file__), "native", "libgpu_picking.so")
    if not os.path.exists(lib):
        import __graft_entry__ as ge
        ge._build_library_test_helpers()
    L = C.CDLL(lib)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.run_picking.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                              dp, C.c_double, dp, ip]
    return L


def test_gpuvbd_drop_in_picks_without_rebuilding():
    """The C++ GpuVBD keeps its solver across the pick / drag / release topology updates (no
    recolouring, retiling or autotuning) and gives the same positions, bit for bit, as the
    handle-level dynamic anchors on the same sequence."""
    from spg_gb300 import scenes as S
    n, steps, start, end, lanes = 33, 10, 2, 7, 4
    obj = S.spring_cloth(n).objects[0]
    v = obj.nv - 5
    gpu = N.VbdSolver([obj], dt=1 / 120, iterations=20, gravity=GRAVITY, kernel=1, lanes_per_vertex=lanes)
    path = np.zeros((steps, 3))
    anchor = None
    for s in range(steps):
        if s == start:
            anchor = gpu.state(0)[0][v].copy()
            path[s] = anchor
        if anchor is not None and s > start:
            anchor = gpu.state(0)[0][v] + np.array([0.002, 0.0, 0.004])
            path[s] = anchor
        if s == end:
            anchor = None
        gpu.set_picks([] if anchor is None else [(0, v, anchor, PICK_K)])
        gpu.step()
    L = _driver()
    out = np.zeros((obj.nv, 3))
    rebuilds = C.c_int()
    rc = L.run_picking(n, 1, lanes, 20, 1 / 120, steps, v, start, end, np.ascontiguousarray(path).ctypes.data_as(
        C.POINTER(C.c_double)), PICK_K, out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rebuilds))
    assert rc == 0
    assert rebuilds.value == 0
    assert np.array_equal(out, gpu.state(0)[0])
