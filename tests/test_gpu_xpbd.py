"""GPU parity of the XPBD colored projection against the FP64 oracle."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")


@pytest.mark.parametrize("scene", ["springs", "cloth", "beam"])
def test_xpbd_positions(scene):
    if scene == "springs":
        obj, dt, sub = scenes.spring_cloth_cfg3(33), 1 / 120, 20
    elif scene == "cloth":
        obj, dt, sub = scenes.cloth_cfg1(17), 1 / 60, 20
    else:
        obj, dt, sub = scenes.beam_cfg2(9, 4, 4), 1 / 60, 20
    gpu = N.XpbdSolver([obj], dt=dt, substeps=sub, gravity=scenes.GRAVITY)
    ref = O.Xpbd(obj, dt, sub, scenes.GRAVITY)
    for e in range(len(obj.energies)):
        assert np.array_equal(gpu.stencil_colors(0, e), ref.stencil_colors(e))
    for _ in range(5):
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    print(f"XPBD {scene}: max position error {err:.3e} m (extent {extent:.3f} m)")
    assert err <= 1e-4 * extent


@pytest.mark.parametrize("kernel", [2, 3])
@pytest.mark.parametrize("scene", ["springs", "springs_odd_step", "cloth", "beam", "membranes"])
def test_persistent_kernels_equal_phase_launches(scene, kernel):
    """The dataflow XPBD kernel (2: every substep in one launch, chunks ordered by their vertex
    chains) and the synchronised one (3: every substep in one launch, a grid barrier between
    phases) perform the same projections in the same per-vertex order as one launch per
    (energy, stencil colour) phase, so positions and velocities agree bit for bit."""
    substeps = 20
    if scene == "springs":
        obj, dt = scenes.spring_cloth_cfg3(129), 1 / 120
    elif scene == "springs_odd_step":  # 1/h and 1/h^2 not exact in FP32
        obj, dt, substeps = scenes.spring_cloth_cfg3(65), 1 / 97, 7
    elif scene == "cloth":
        obj, dt = scenes.cloth_cfg1(33), 1 / 60
    elif scene == "beam":
        obj, dt = scenes.beam_cfg2(11, 4, 4), 1 / 60
    else:
        obj, dt = scenes.cloth_variant((O.CHOI_MEMBRANE, O.QUAD_BENDING), 17), 1 / 60
    kw = dict(dt=dt, substeps=substeps, gravity=scenes.GRAVITY)
    a = N.XpbdSolver([obj], kernel=1, **kw)
    b = N.XpbdSolver([obj], kernel=kernel, **kw)
    for _ in range(3):
        a.step()
        b.step()
    xa, va = a.state(0)
    xb, vb = b.state(0)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


@pytest.mark.parametrize("kernel", [2, 3])
def test_persistent_kernels_batch_of_objects(kernel):
    """Several objects in one persistent launch, each against its own oracle instance."""
    objs = scenes.patch_batch_cfg4(5, 8, 16, seed=3)
    gpu = N.XpbdSolver(objs, dt=1 / 60, substeps=10, gravity=scenes.GRAVITY, kernel=kernel)
    refs = [O.Xpbd(o, 1 / 60, 10, scenes.GRAVITY) for o in objs]
    for _ in range(3):
        gpu.step()
        for r in refs:
            r.step()
    for k, r in enumerate(refs):
        assert np.abs(gpu.state(k)[0] - r.state()[0]).max() <= 1e-4
