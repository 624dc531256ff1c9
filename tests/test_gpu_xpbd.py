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
