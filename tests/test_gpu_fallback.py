"""The FP64 3x3 block solve taken when a vertex block's condition estimate exceeds the
threshold (SpgxVbdParams.fallback_condition, default 1e6), against the FP64 oracle
(vbd.cpp:139-146: x += H^-1 f when det H > 1e-10)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")


def rope(n=64, length=1.0, k=1e4, mass=1e-6):
    """A straight rope of n vertices along x with springs between neighbours and both ends
    anchored. At rest a vertex block is m/h^2 I + 2 k x x^T: with m = 1e-6 kg, k = 1e4 N/m and
    h = 1/60 s its condition number is 1 + 2 k h^2 / m = 5.6e6, above the 1e6 threshold, with
    the small eigenvalues across the rope, where gravity pulls."""
    x = np.zeros((n, 3))
    x[:, 0] = np.linspace(0.0, length, n)
    L0 = length / (n - 1)
    springs = np.stack([np.arange(n - 1), np.arange(1, n)], axis=1).astype(np.int32)
    sp = np.tile([L0, k, 1.0 / k], (n - 1, 1))
    ends = np.array([[0], [n - 1]], np.int32)
    an = np.array([[*x[0], 1e5, 1e-5], [*x[-1], 1e5, 1e-5]])
    energies = [O.Energy(O.SPRING, springs, sp), O.Energy(O.ANCHOR, ends, an)]
    return O.SceneObject(x.copy(), np.full(n, mass), energies, None, x.copy())


@pytest.mark.parametrize("kernel", [1, 3])
def test_ill_conditioned_blocks_take_the_fp64_solve(kernel):
    obj = rope()
    g = scenes.GRAVITY
    ref = O.Vbd(obj, 1 / 60, 1, 20, g, O.VERTEX_AD)
    fb = N.VbdSolver([obj], dt=1 / 60, iterations=20, gravity=g, kernel=kernel)
    fp32 = N.VbdSolver([obj], dt=1 / 60, iterations=20, gravity=g, kernel=kernel, fallback_condition=1e30)
    fallbacks = 0
    for _ in range(10):
        ref.step()
        fallbacks += fb.step().fallback_solves
        assert fp32.step().fallback_solves == 0
    xr, _ = ref.state()
    e_fb = float(np.abs(fb.state(0)[0] - xr).max())
    e_32 = float(np.abs(fp32.state(0)[0] - xr).max())
    print(f"rope, kernel {kernel}: {fallbacks} FP64 solves in 10 steps; max |x - x64| with the fallback "
          f"{e_fb:.3e} m, FP32 solves only {e_32:.3e} m; sag {-xr[:, 2].min():.4e} m")
    assert fallbacks > 0
    assert e_fb <= 1e-4 * 1.0


@pytest.mark.parametrize("kernel", [0, 3])
def test_every_block_in_fp64_matches_the_fp32_path(kernel):
    """The 33x33 StVK cloth (100 iterations, 10 steps) with the threshold at 1, below any
    block's condition estimate, so every solve runs in FP64: within 1e-4 of the extent of the
    oracle, and within the FP32 element error of the FP32 solves."""
    obj = scenes.cloth_cfg1()
    kw = dict(dt=1 / 60, iterations=100, gravity=scenes.GRAVITY, kernel=kernel)
    fb = N.VbdSolver([obj], fallback_condition=1.0, **kw)
    plain = N.VbdSolver([obj], **kw)
    ref = O.Vbd(obj, 1 / 60, 1, 100, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(10):
        st = fb.step()
        assert st.fallback_solves == obj.nv * 100
        assert plain.step().fallback_solves == 0
        ref.step()
    xf, xp, xr = fb.state(0)[0], plain.state(0)[0], ref.state()[0]
    extent = float(np.ptp(obj.x0, axis=0).max())
    e_ref, e_32 = float(np.abs(xf - xr).max()), float(np.abs(xf - xp).max())
    print(f"cfg1 all-FP64 solves, kernel {fb.launch()}: max |x - x64| {e_ref:.3e} m, max |x - x_fp32 solves| "
          f"{e_32:.3e} m, FP32 solves vs oracle {float(np.abs(xp - xr).max()):.3e} m")
    assert e_ref <= 1e-4 * extent
    assert e_32 <= 1e-5 * extent
