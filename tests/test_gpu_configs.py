"""GPU parity at the benchmark configurations' full sizes, against the FP64 oracle.

- 41x11x11 Stable Neo-Hookean bar (4,961 vertices, 24,000 tets), 50 iterations, 20 steps;
- 513x513 jittered spring cloth (263,169 vertices), 20 iterations, 3 steps, plus the
  FP64-reduced residual;
- the 512-patch StVK batch (3.02 M vertices in one solver), one step of 30 iterations, with
  every fourth patch checked against its own oracle instance (128 patches).

Positions must agree to 1e-4 of the scene's extent. Each oracle run is shared by the kernels
tested against it.
"""
import functools

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

N = pytest.importorskip("spg_gb300.native")


@functools.lru_cache(maxsize=None)
def _bar_oracle():
    obj = scenes.beam_cfg2()
    ref = O.Vbd(obj, 1 / 60, 1, 50, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(20):
        ref.step()
    return obj, ref.state()[0]


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
def test_snh_bar_41x11x11_20_steps(kernel):
    obj, xr = _bar_oracle()
    assert obj.nv == 4961 and sum(e.n for e in obj.energies if e.type == O.SNH) == 24000
    gpu = N.VbdSolver([obj], dt=1 / 60, iterations=50, gravity=scenes.GRAVITY, kernel=kernel)
    for _ in range(20):
        gpu.step()
    xg, _ = gpu.state(0)
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    print(f"SNH bar 41x11x11, 20 steps, kernel {gpu.launch()}: max |x - x64| {err:.3e} m "
          f"(extent {extent:.3f} m, tip sag {obj.x0[:, 2].min() - xr[:, 2].min():.4e} m)")
    assert err <= 1e-4 * extent


@functools.lru_cache(maxsize=None)
def _cloth_oracle():
    obj = scenes.spring_cloth_cfg3(513)
    ref = O.Vbd(obj, 1 / 120, 1, 20, scenes.GRAVITY, O.VERTEX_AD)
    xs, res = [], []
    for _ in range(3):
        ref.step()
        xs.append(ref.state()[0])
        res.append(ref.residual())
    return obj, xs, res


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
def test_spring_cloth_513_positions_and_residual(kernel):
    obj, xs, res = _cloth_oracle()
    assert obj.nv == 263169
    gpu = N.VbdSolver([obj], dt=1 / 120, iterations=20, gravity=scenes.GRAVITY, kernel=kernel)
    extent = float(np.ptp(obj.x0, axis=0).max())
    for s in range(3):
        gpu.step()
        xg, _ = gpu.state(0)
        err = float(np.abs(xg - xs[s]).max())
        rg = gpu.residual()
        print(f"513 cloth step {s + 1}, kernel {gpu.launch()}: max |x - x64| {err:.3e} m (extent {extent:.3f} m); "
              f"residual GPU {rg:.6e} oracle {res[s]:.6e} (rel diff {abs(rg - res[s]) / res[s]:.2e})")
        assert err <= 1e-4 * extent
        assert abs(rg - res[s]) <= 1e-3 * res[s]


@functools.lru_cache(maxsize=None)
def _batch_oracle():
    from tests.oracle_pool import solve_many
    objs = scenes.patch_batch_cfg4(512)
    checked = list(range(0, 512, 4))
    out = solve_many([objs[i] for i in checked], 1 / 60, 30, 1, scenes.GRAVITY, perturb=1e-9)
    return objs, checked, [x for x, _ in out], [s for _, s in out]


@pytest.mark.parametrize("kernel", [0, 1, 3])
def test_patch_batch_512_one_step(kernel):
    """The whole 512-patch batch in one solver; every fourth patch against its own FP64 oracle
    instance. The reference's VBD (full element Hessians, no definiteness projection) is
    unstable on a few patches of this generator: there the FP64 oracle itself moves by
    millimetres to centimetres when its start positions move by 1e-9 m, so no precision can
    track it. A patch counts as well conditioned when that response stays below 1e-6 m (an
    amplification of at most 1000); every well-conditioned patch must agree to 1e-4 of its
    1 m extent, and they must be at least 90 % of the patches checked."""
    objs, checked, xs, sens = _batch_oracle()
    nv = [o.nv for o in objs]
    assert len(objs) == 512 and min(int(round(np.sqrt(n))) for n in nv) >= 16 and max(nv) <= 128 * 128
    gpu = N.VbdSolver(objs, dt=1 / 60, iterations=30, gravity=scenes.GRAVITY, kernel=kernel)
    gpu.step()
    worst, excluded = 0.0, []
    for i, xr, s in zip(checked, xs, sens):
        xg, _ = gpu.state(i)
        assert np.all(np.isfinite(xg))
        err = float(np.abs(xg - xr).max())
        if s > 1e-6:
            excluded.append((i, int(round(np.sqrt(nv[i]))), s, err))
            continue
        worst = max(worst, err)
    good = len(checked) - len(excluded)
    print(f"512-patch batch ({sum(nv)} vertices), kernel {gpu.launch()}: worst max |x - x64| over {good} "
          f"well-conditioned patches {worst:.3e} m (extent 1 m); ill-conditioned (patch, side, FP64 response "
          f"to 1e-9 m, GPU difference): {[(i, n, f'{s:.1e}', f'{e:.1e}') for i, n, s, e in excluded]}")
    assert good >= 0.9 * len(checked)
    assert worst <= 1e-4
