"""GPU parity of the VBD path against the FP64 oracle (run on a GB300)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

pytestmark = pytest.mark.gpu

N = pytest.importorskip("spg_gb300.native")


def _f32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def _deformed(obj, steps, iters, dt=1 / 60):
    s = O.Vbd(obj, dt, 1, iters, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(steps):
        s.step()
    o = obj.copy()
    o.x, _ = s.state()
    return o


U32 = 2.0 ** -24  # FP32 unit roundoff


def _element_samples(obj, rng, positions, jitter_rel, n_per_energy=200):
    """(type, X, params) of random elements of every energy, at `positions` moved by a random
    displacement of relative size jitter_rel() of the element size."""
    out = []
    for e in obj.energies:
        idx = rng.integers(0, e.n, size=min(n_per_energy, e.n))
        for i in idx:
            X = positions[e.stencils[i]].copy()
            ell = max(float(np.ptp(X, axis=0).max()), 1e-3)
            X += rng.normal(size=X.shape) * ell * jitter_rel()
            out.append((e.type, _f32(X), _f32(e.params[i])))
    return out


def _element_errors(samples):
    """Per energy type and element: every vertex block of the element on the GPU (FP32)
    against the oracle's full-element FP64 AD (the reference's TinyAD path). Returns arrays of
    eg = |g - g64| / |g64| over the element's whole gradient, egb = |g - g64| /
    (1e-5 |g64| + 8 u |H64| l) (u the FP32 unit roundoff, l the element size) and
    eh = |H_blocks - H64_blocks| / |H64| (Frobenius, the element's diagonal blocks against its
    whole Hessian)."""
    out = {}
    for etype in sorted({s[0] for s in samples}):
        sub = [s for s in samples if s[0] == etype]
        S = O.STENCIL_SIZE[etype]
        X = np.repeat(np.stack([s[1].reshape(-1) for s in sub]), S, axis=0)
        P = np.repeat(np.stack([s[2] for s in sub]), S, axis=0)
        slots = np.tile(np.arange(S), len(sub))
        g, H = N.eval_vertex_blocks(etype, X, P, slots)
        g = g.reshape(len(sub), 3 * S)
        H = H.reshape(len(sub), S, 3, 3)
        eg, egb, eh = [], [], []
        for k, (_, Xk, Pk) in enumerate(sub):
            gr, Hr = O.element_full(etype, Xk, Pk)
            ell = float(np.ptp(Xk.reshape(-1, 3), axis=0).max()) if S > 1 else 1.0
            d = np.linalg.norm(g[k] - gr)
            nH = np.linalg.norm(Hr)
            eg.append(d / max(np.linalg.norm(gr), 1e-300))
            egb.append(d / max(1e-5 * np.linalg.norm(gr) + 8 * U32 * nH * ell, 1e-300))
            dH = sum(np.linalg.norm(H[k, j] - Hr[3 * j:3 * j + 3, 3 * j:3 * j + 3]) ** 2 for j in range(S))
            eh.append(np.sqrt(dH) / max(nH, 1e-300))
        out[etype] = (np.array(eg), np.array(egb), np.array(eh))
    return out


def _scene(name):
    if name == "cloth":
        return scenes.cloth_cfg1(17), 1 / 60
    if name == "beam":
        return scenes.beam_cfg2(9, 4, 4), 1 / 60
    return scenes.spring_cloth_cfg3(33), 1 / 120


@pytest.mark.parametrize("scene", ["cloth", "beam", "springs"])
def test_element_blocks_match_tinyad_fp64(scene):
    """Per-element parity of the FP32 device blocks with the oracle's FP64 full-element AD on
    the same FP32 inputs, every sampled element checked (the maximum, not a quantile), on
    strained elements (the scene after 3 steps, jittered by 0.2 % of its extent) and near-rest
    elements (rest positions moved by 1e-6 to 1e-2 of the element size).

    - Hessians: the element's vertex blocks within 1e-5 of the element's Hessian (Frobenius).
    - Springs and anchors: the element gradient within 1e-5 relative. The spring stretch
      l - L0 is formed without cancellation, so this holds down to strains of 1e-6.
    - Bending, StVK and Stable Neo-Hookean: their gradients vanish at rest, where an FP32
      evaluation is a difference of terms of the size of |H| l (the FP32 dihedral angle alone
      is resolved to about 1e-7 rad). They are held to 1e-5 relative plus 8 FP32 roundoffs of
      that scale: |dg| <= 1e-5 |g| + 8 u |H| l, i.e. 1e-5 relative once the strain exceeds
      about 5 %, and a few roundoffs of |H| l below it."""
    rng = np.random.default_rng(7)
    obj, dt = _scene(scene)
    deformed = _deformed(obj, 3, 20, dt=dt)
    extent_rel = 2e-3 * float(np.ptp(obj.x))
    sets = {"strained": _element_samples(deformed, rng, deformed.x, lambda: 0.0),
            "near-rest": _element_samples(obj, rng, obj.x0, lambda: 10.0 ** rng.uniform(-6, -2))}
    # strained: the deformed scene plus an absolute jitter of 0.2 % of the extent
    sets["strained"] = [(t, _f32(X + rng.normal(scale=extent_rel, size=X.shape)), p)
                        for t, X, p in sets["strained"]]
    for name, samples in sets.items():
        for etype, (eg, egb, eh) in _element_errors(samples).items():
            print(f"{scene} {name} type {etype}: element grad rel max {eg.max():.2e} (median {np.median(eg):.1e}), "
                  f"bound use max {egb.max():.2f}; hess max {eh.max():.2e}")
            assert eh.max() <= 1e-5
            if etype in (O.SPRING, O.ANCHOR):
                assert eg.max() <= 1e-5
            else:
                assert egb.max() <= 1.0


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_cloth_cfg1_positions_after_10_steps(kernel):
    """33x33 StVK cloth, 100 iterations/step, 10 steps: |x_gpu - x_fp64| <= 1e-4 extent."""
    obj = scenes.cloth_cfg1()
    gpu = N.VbdSolver([obj], dt=1 / 60, iterations=100, gravity=scenes.GRAVITY, kernel=kernel)
    ref = O.Vbd(obj, 1 / 60, 1, 100, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(10):
        gpu.step()
        ref.step()
    xg, vg = gpu.state(0)
    xr, vr = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    print(f"cfg1 max position error {err:.3e} m (extent {extent} m), sag {xr[:, 2].min():.4f} m")
    assert err <= 1e-4 * extent


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_spring_cloth_positions_after_10_steps(kernel):
    obj = scenes.spring_cloth_cfg3(65)
    gpu = N.VbdSolver([obj], dt=1 / 120, iterations=20, gravity=scenes.GRAVITY, kernel=kernel)
    ref = O.Vbd(obj, 1 / 120, 1, 20, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(10):
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    print(f"spring cloth max position error {err:.3e} m (extent {extent:.3f} m)")
    assert err <= 1e-4 * extent


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_snh_beam_positions(kernel):
    obj = scenes.beam_cfg2(11, 4, 4)
    gpu = N.VbdSolver([obj], dt=1 / 60, iterations=50, gravity=scenes.GRAVITY, kernel=kernel)
    ref = O.Vbd(obj, 1 / 60, 1, 50, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(10):
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    print(f"SNH beam max position error {err:.3e} m (extent {extent:.3f} m)")
    assert err <= 1e-4 * extent


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_batch_matches_independent_solvers(kernel):
    objs = scenes.patch_batch_cfg4(6, 8, 20, seed=3)
    gpu = N.VbdSolver(objs, dt=1 / 60, iterations=30, gravity=scenes.GRAVITY, kernel=kernel)
    refs = [O.Vbd(o, 1 / 60, 1, 30, scenes.GRAVITY, O.VERTEX_AD) for o in objs]
    for _ in range(3):
        gpu.step()
        for r in refs:
            r.step()
    for k, r in enumerate(refs):
        xg, _ = gpu.state(k)
        xr, _ = r.state()
        assert np.abs(xg - xr).max() <= 1e-4


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_residual_matches_oracle(kernel):
    """FP64-reduced residual ||M/h^2 (x - y) + grad E(x)|| of the GPU state against the
    oracle's at the same state and inertial target."""
    obj = scenes.cloth_cfg1(17)
    gpu = N.VbdSolver([obj], dt=1 / 60, iterations=0, gravity=scenes.GRAVITY, kernel=kernel)
    ref = O.Vbd(obj, 1 / 60, 1, 0, scenes.GRAVITY, O.VERTEX_AD)
    # Before any step the target is x itself: the residual is ||grad E(x)||.
    assert abs(gpu.residual() - ref.residual()) <= 1e-4 * ref.residual() + 1e-6
    # Steps without iterations leave x = y, and the inertia term vanishes again; with
    # iterations the inertia term enters too.
    for iters in (0, 3):
        gpu.set_params(iterations=iters)
        ref2 = O.Vbd(obj, 1 / 60, 1, iters, scenes.GRAVITY, O.VERTEX_AD)
        g2 = N.VbdSolver([obj], dt=1 / 60, iterations=iters, gravity=scenes.GRAVITY, kernel=kernel)
        g2.step()
        ref2.step()
        rg, rr = g2.residual(), ref2.residual()
        print(f"iterations {iters}: residual gpu {rg:.6e} oracle {rr:.6e}")
        assert abs(rg - rr) <= 1e-3 * rr + 1e-6


def test_colors_and_adjacency_through_handle():
    obj = scenes.cloth_cfg1(33)
    gpu = N.VbdSolver([obj], dt=1 / 60, iterations=1, gravity=scenes.GRAVITY)
    ref = O.Vbd(obj, 1 / 60, 1, 1, scenes.GRAVITY)
    assert np.array_equal(gpu.colors(0), ref.colors())
    c1, e1 = gpu.adjacency(0)
    c2, e2 = ref.adjacency(len(obj.energies))
    assert np.array_equal(c1, c2) and np.array_equal(e1, e2)


@pytest.mark.parametrize("lanes,tile", [(1, 64), (2, 64), (4, 64), (4, 32), (2, 32), (4, 16), (8, 16)])
def test_dataflow_kernel_equals_colour_launches(lanes, tile):
    """The dataflow kernel runs the same Gauss-Seidel order as one launch per colour, so with
    the same lanes per vertex (same per-vertex summation order) it gives the same positions
    bit for bit, over steps of 20 sweeps and for a tolerance-mode step."""
    from spg_gb300 import scenes as S
    obj = S.spring_cloth(129).objects[0]
    kw = dict(dt=1 / 120, iterations=20, gravity=scenes.GRAVITY, lanes_per_vertex=lanes, tile_vertices=tile)
    a = N.VbdSolver([obj], kernel=2, **kw)
    b = N.VbdSolver([obj], kernel=3, **kw)
    assert a.launch() == (2, lanes, tile * lanes) and b.launch() == (3, lanes, tile * lanes)
    for _ in range(3):
        a.step()
        b.step()
    assert np.array_equal(a.state(0)[0], b.state(0)[0])
    a.set_params(tolerance=1e-4, max_iterations=400, check_interval=50)
    b.set_params(tolerance=1e-4, max_iterations=400, check_interval=50)
    sa, sb = a.step(), b.step()
    assert sa.iterations == sb.iterations
    assert np.array_equal(a.state(0)[0], b.state(0)[0])


@pytest.mark.parametrize("kernel", [0, 2, 3])
def test_autotuned_tile_size(kernel):
    """With no tile size requested the autotuner tries 32- and 64-vertex tiles and leaves the
    scene tiled for its pick: the solver then steps exactly as one created with that size."""
    from spg_gb300 import scenes as S
    obj = S.spring_cloth(129).objects[0]
    kw = dict(dt=1 / 120, iterations=20, gravity=scenes.GRAVITY)
    a = N.VbdSolver([obj], kernel=kernel, **kw)
    k, g, b = a.launch()
    if k == 1:
        pytest.skip("the lanes kernel won on this device")
    assert k in (2, 3) and b // g in (32, 64) and b % g == 0
    ref = N.VbdSolver([obj], kernel=k, lanes_per_vertex=g, tile_vertices=b // g, **kw)
    assert ref.launch() == (k, g, b)
    for _ in range(3):
        a.step()
        ref.step()
    assert np.array_equal(a.state(0)[0], ref.state(0)[0])


@pytest.mark.parametrize("solver", ["vbd", "xpbd"])
def test_pinned_and_pageable_host_state_agree(solver):
    """State moved through host arrays pinned by CUDA (asynchronous copies) and through
    pageable arrays gives the same device state and the same host arrays, bit for bit."""
    torch = pytest.importorskip("torch")
    obj = scenes.spring_cloth_cfg3(65)
    nv = obj.x.shape[0]
    rng = np.random.default_rng(7)
    x = obj.x + rng.normal(scale=1e-3, size=obj.x.shape)
    v = rng.normal(scale=1e-2, size=obj.x.shape)
    if solver == "vbd":
        make = lambda: N.VbdSolver([obj], dt=1 / 120, iterations=20, gravity=scenes.GRAVITY)  # noqa: E731
    else:
        make = lambda: N.XpbdSolver([obj], dt=1 / 120, substeps=10, gravity=scenes.GRAVITY)  # noqa: E731
    a, b = make(), make()
    xp = torch.empty((nv, 3), dtype=torch.float64, pin_memory=True).numpy()
    vp = torch.empty((nv, 3), dtype=torch.float64, pin_memory=True).numpy()
    xp[:] = x
    vp[:] = v
    a.set_state(0, x, v)
    b.set_state(0, xp, vp)
    for _ in range(3):
        a.step()
        b.step()
    xa, va = a.state(0)
    xp.fill(np.nan)
    vp.fill(np.nan)
    b.get_state_into(0, xp, vp)
    assert np.array_equal(xa, xp) and np.array_equal(va, vp)
