"""Implicit Euler (one Newton step per substep, the reference's ImplicitEulerNewtonDx): the
FP64 oracle's conjugate-gradient restatement against a direct solve (CPU), and the GPU
solver against the oracle on scenes with every energy type (GB300). Continuum springs run on
a 3D truss: on a flat cloth at rest the implicit step is nearly singular out of plane, and a
1e-9 m perturbation grows to millimetres in one step in the FP64 oracle itself."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import implicit_ref as IR
from oracle import pyoracle as O
from tests import scenes


def _scenes():
    return {
        "stvk_cloth": scenes.cloth_cfg1(9),
        "snh_beam": scenes.beam_cfg2(5, 3, 3),
        "spring_cloth": scenes.spring_cloth_cfg3(9),
        "stvk_tet_load": scenes.beam_tet_variant(O.STVK_TET, nx=5, ny=3, nz=3, load=True),
        "bw": scenes.cloth_variant((O.BW_MEMBRANE, O.BW_BENDING), rows=7),
        "choi_quad": scenes.cloth_variant((O.CHOI_MEMBRANE, O.QUAD_BENDING), rows=7),
        "truss": scenes.truss_variant(),
    }


def test_oracle_cg_matches_direct_solve():
    rng = np.random.default_rng(0)
    n = 60
    B = sp.random(n, n, density=0.1, random_state=1)
    A = (B @ B.T + sp.eye(n) * 2.0).tocsr()
    b = rng.normal(size=n)
    x, it, rel = IR.conjugate_gradient(A, b, tol=1e-10, max_iterations=1000)
    assert rel < 1e-10 and 0 < it <= 1000
    assert np.allclose(x, spla.spsolve(A.tocsc(), b), rtol=1e-8, atol=1e-10)


def _chronopoulos_gear_cg(A, b, tol=1e-5, max_iterations=300):
    """The recurrences of the GPU solve (implicit_cg.cuh), restated in FP64: u = D^-1 r,
    w = A u, gamma = r.u, delta = u.w, beta = gamma / gamma_prev,
    alpha = gamma / (delta - beta gamma / alpha_prev), p = u + beta p, s = w + beta s,
    x += alpha p, r -= alpha s; the stopping test after each update."""
    n = b.shape[0]
    x, p, s = np.zeros(n), np.zeros(n), np.zeros(n)
    rhs2 = float(b @ b)
    d = A.diagonal()
    inv = np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 1.0)
    thr = max(tol * tol * rhs2, np.finfo(float).tiny)
    r = b.copy()
    u = inv * r
    its, gamma_prev, alpha_prev = 0, 0.0, 1.0
    for k in range(max_iterations + 1):
        w = A @ u
        gamma, rr, delta = float(r @ u), float(r @ r), float(u @ w)
        if k == 0:
            if rhs2 == 0.0 or rr < thr:
                break
        else:
            its += 1
            if rr < thr or its >= max_iterations:
                break
        beta = 0.0 if k == 0 else gamma / gamma_prev
        alpha = gamma / (delta - beta * gamma / alpha_prev)
        p = u + beta * p
        s = w + beta * s
        x += alpha * p
        r -= alpha * s
        u = inv * r
        gamma_prev, alpha_prev = gamma, alpha
    return x, its, np.sqrt(rr / rhs2) if rhs2 else 0.0


def test_chronopoulos_gear_recurrences_match_the_reference_cg():
    """The GPU solve's form of preconditioned CG (one reduction per iteration) takes the same
    iterates as Eigen's (the oracle's restatement): on random SPD systems with a spread of
    diagonal scales (condition numbers near 4e4), the same iteration count, and solutions within
    1e-10 relative when the solve converges."""
    rng = np.random.default_rng(3)
    for n, density in ((60, 0.1), (200, 0.03), (500, 0.01)):
        B = sp.random(n, n, density=density, random_state=int(rng.integers(1 << 30)))
        D = sp.diags(10.0 ** rng.uniform(-1, 1, size=n))
        A = (D @ (B @ B.T + sp.eye(n) * 0.5) @ D).tocsr()
        b = rng.normal(size=n)
        for tol, cap in ((1e-8, 1000), (1e-5, 20)):
            x_ref, it_ref, rel_ref = IR.conjugate_gradient(A, b, tol=tol, max_iterations=cap)
            x_cg, it_cg, rel_cg = _chronopoulos_gear_cg(A, b, tol=tol, max_iterations=cap)
            assert it_cg == it_ref, (n, tol, it_cg, it_ref)
            err = np.abs(x_cg - x_ref).max() / np.abs(x_ref).max()
            if it_ref < cap:  # converged: both residuals under the tolerance, the same x
                assert rel_cg < tol and rel_ref < tol
                assert err <= 1e-10, (n, tol, err)
            else:  # stopped by the cap mid-solve, where rounding has grown (measured <= 4e-9)
                assert err <= 1e-7, (n, tol, err)
                assert abs(rel_cg - rel_ref) <= 1e-2 * rel_ref


def test_oracle_steps_every_scene():
    for name, obj in _scenes().items():
        s = IR.ImplicitEuler(obj, 1 / 60, 1, scenes.GRAVITY)
        for _ in range(2):
            s.step()
        x, _ = s.state()
        assert np.all(np.isfinite(x)), name


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["stvk_cloth", "snh_beam", "spring_cloth", "stvk_tet_load", "bw", "choi_quad",
                                  "truss"])
def test_positions_after_10_steps_match_oracle(name):
    N = pytest.importorskip("spg_gb300.native")
    obj = _scenes()[name]
    gpu = N.ImplicitSolver([obj], dt=1 / 60, substeps=1, gravity=scenes.GRAVITY)
    ref = IR.ImplicitEuler(obj, 1 / 60, 1, scenes.GRAVITY)
    its = []
    for _ in range(10):
        st = gpu.step()
        ref.step()
        its.append((int(st.iterations), ref.last_iterations))
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = np.abs(xg - xr).max()
    print(f"implicit {name}: max |dx| after 10 steps {err:.3g} m (extent {extent:.3g} m); CG iterations "
          f"GPU/oracle {its[:3]}")
    assert err <= 1e-4 * extent


def _bent_spring_cloth():
    """9x9 spring cloth (k 1e3) with stiff discrete bending (k 0.03), started from a 1 cm
    out-of-plane wave: bending drives the motion (without it the cloth ends 8 cm elsewhere
    after three steps), and the C hess(theta) term of its Hessian is far from zero."""
    obj = O.build_spring_cloth(0.1 * 0.25, 0.5, 0.5, 9, 9, 1e3, 0.03, 1e5, 0.1, 3)
    x0 = obj.x0
    u = (x0[:, 0] - x0[:, 0].min()) / np.ptp(x0[:, 0])
    v = (x0[:, 1] - x0[:, 1].min()) / np.ptp(x0[:, 1])
    obj.x = x0 + np.stack([0 * u, 0 * u, 0.01 * np.sin(np.pi * u) * np.sin(2 * np.pi * v)], 1)
    return obj


@pytest.mark.gpu
def test_bending_dominated_cloth_matches_oracle():
    """The closed-form spring and bending assembly (forward mode on the analytic dihedral
    gradient) against the oracle's full-element automatic differentiation."""
    N = pytest.importorskip("spg_gb300.native")
    obj = _bent_spring_cloth()
    gpu = N.ImplicitSolver([obj], dt=1 / 60, substeps=1, gravity=scenes.GRAVITY)
    ref = IR.ImplicitEuler(obj, 1 / 60, 1, scenes.GRAVITY)
    for _ in range(5):
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    err = float(np.abs(xg - xr).max())
    moved = float(np.abs(xr - obj.x).max())
    print(f"bent spring cloth: max |dx| {err:.3g} m after 5 steps (moved {moved:.3g} m)")
    assert err <= 1e-3 * moved


@pytest.mark.gpu
def test_wide_system_runs_fp64_products():
    """Masses and stiffnesses of the truss scaled by 1e20: the system matrix exceeds the
    double-float range (2^60), so every CG solve's products run in FP64 (reported in
    warm_accepted). The motion is the unscaled truss's, and matches the oracle's."""
    N = pytest.importorskip("spg_gb300.native")
    S = 1e20
    base = scenes.truss_variant()
    wide = scenes.truss_variant(k_cont=2e3 * S, k_sq=5e2 * S)
    wide.mass = wide.mass * S
    for e in wide.energies:
        if e.type == O.ANCHOR:
            e.params[:, 3] *= S
    g_wide = N.ImplicitSolver([wide], dt=1 / 60, substeps=1, gravity=scenes.GRAVITY)
    g_base = N.ImplicitSolver([base], dt=1 / 60, substeps=1, gravity=scenes.GRAVITY)
    ref = IR.ImplicitEuler(wide, 1 / 60, 1, scenes.GRAVITY)
    for _ in range(5):
        assert g_wide.step().warm_accepted == 1
        assert g_base.step().warm_accepted == 0
        ref.step()
    xw, xb, xr = g_wide.state(0)[0], g_base.state(0)[0], ref.state()[0]
    moved = float(np.abs(xr - wide.x).max())
    assert np.abs(xw - xr).max() <= 1e-3 * moved
    assert np.abs(xw - xb).max() <= 1e-3 * moved


def _pinned_spring_cloth(n):
    """A spring cloth with the large-cloth spacing (2 m at 513 vertices per side, k 1e4, no
    jitter) under a soft pin (k 50) at every vertex, started from a 1 cm out-of-plane wave:
    every spring is stretched, so the Newton system is positive definite and the FP64 oracle
    well conditioned (a 1e-9 m perturbation of the start moves its result by 3e-10 m; about 60
    CG iterations per step). 66,049 rows at n = 257, above the 65,536 from which the CG takes
    4 lanes per row."""
    w = 2.0 * (n - 1) / 512
    obj = O.build_spring_cloth(0.1 * w * w, w, w, n, n, 1e4, 1e-4, 1e5, 0.0, 7)
    nv = obj.x.shape[0]
    pins = np.concatenate([obj.x0, np.full((nv, 1), 50.0), np.full((nv, 1), 1 / 50.0)], axis=1)  # [a, k, 1/k]
    obj.energies.append(scenes._energy(O.ANCHOR, np.arange(nv, dtype=np.int32).reshape(-1, 1), pins))
    obj.x = obj.x0 + np.stack([np.zeros(nv), np.zeros(nv), 0.01 * np.sin(3.0 * obj.x0[:, 0])], 1)
    return obj


@pytest.mark.gpu
@pytest.mark.slow
def test_large_system_matches_oracle():
    """The double-float CG with 4 lanes per row (symmetric product, reverse Cuthill-McKee rows)
    against the FP64 oracle, two steps of the pinned 257x257 cloth."""
    N = pytest.importorskip("spg_gb300.native")
    obj = _pinned_spring_cloth(257)
    assert obj.x.shape[0] >= 65536
    gpu = N.ImplicitSolver([obj], dt=1 / 120, substeps=1, gravity=scenes.GRAVITY)
    ref = IR.ImplicitEuler(obj, 1 / 120, 1, scenes.GRAVITY)
    its = []
    for _ in range(2):
        st = gpu.step()
        ref.step()
        its.append((int(st.iterations), ref.last_iterations))
        assert st.warm_accepted == 0  # the double-float solve, not the FP64 fallback
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    moved = float(np.abs(xr - obj.x).max())
    err = float(np.abs(xg - xr).max())
    print(f"pinned 257x257 cloth: max |dx| {err:.3g} m after 2 steps (moved {moved:.3g} m); CG iterations "
          f"GPU/oracle {its}")
    assert err <= 1e-4 * moved
    for a, b in its:
        assert abs(a - b) <= max(2, b // 20)


@pytest.mark.gpu
@pytest.mark.slow
def test_double_float_cg_matches_fp64_cg_at_513():
    """The pinned cloth at 513x513 (263,169 vertices, the benchmark cloth's size): two Newton-Dx
    steps with the double-float CG against the same steps with the FP64 CG (cg_precision 1).
    At this size a thread of the CG launch owns more degrees of freedom than it keeps in
    registers, so the direction's memory path runs as well."""
    N = pytest.importorskip("spg_gb300.native")
    obj = _pinned_spring_cloth(513)
    out = []
    for prec in (0, 1):
        gpu = N.ImplicitSolver([obj], dt=1 / 120, substeps=1, gravity=scenes.GRAVITY, cg_precision=prec)
        its = [(int(st.iterations), int(st.warm_accepted)) for st in (gpu.step(), gpu.step())]
        out.append((gpu.state(0)[0], its))
        gpu.close()
    (x_df, it_df), (x_64, it_64) = out
    moved = float(np.abs(x_64 - obj.x).max())
    err = float(np.abs(x_df - x_64).max())
    print(f"pinned 513x513 cloth, two steps: double-float vs FP64 CG max |dx| {err:.3g} m (moved {moved:.3g} m); "
          f"(iterations, FP64 solves) {it_df} / {it_64}")
    assert [w for _, w in it_df] == [0, 0] and [w for _, w in it_64] == [1, 1]
    assert err <= 1e-4 * moved
    for (a, _), (b, _) in zip(it_df, it_64):
        assert a < 300 and abs(a - b) <= max(2, b // 20)


# ---------------------------------------------------------------------------------------
# The other global solvers (NewtonDv, NewtonRobust, BaraffWitkin, BDF2, StaticNewton,
# QuasiStaticNewton, QuasiStaticNewtonRobust, SimplecticEuler), each on scenes where the
# FP64 oracle itself is well conditioned (a 1e-9 m perturbation of the start stays below
# 1e-8 m after 10 steps). The robust methods also run on the StVK cloth, where their step
# control rejects substeps and shrinks the step: the GPU must take the same decisions.

def _method_cases():
    cases = []
    for m in (IR.NEWTON_DV, IR.BARAFF_WITKIN, IR.BDF2, IR.STATIC_NEWTON, IR.QUASI_STATIC_NEWTON):
        cases += [(m, "snh_beam"), (m, "truss")]
    for m in (IR.NEWTON_ROBUST, IR.QUASI_STATIC_NEWTON_ROBUST):
        cases += [(m, "snh_beam"), (m, "stvk_cloth")]
    cases += [(IR.SYMPLECTIC_EULER, "snh_beam"), (IR.SYMPLECTIC_EULER, "truss")]
    return cases


def test_oracle_methods_step():
    obj = _scenes()["snh_beam"]
    for m in range(9):
        dt = 1e-4 if m == IR.SYMPLECTIC_EULER else 1 / 60
        s = IR.ImplicitSolver(obj, dt, 1, scenes.GRAVITY, m)
        s.step()
        x, v = s.state()
        assert np.all(np.isfinite(x)) and np.abs(x - obj.x).max() > 0, m


@pytest.mark.gpu
@pytest.mark.parametrize("method,name", _method_cases())
def test_methods_match_oracle(method, name):
    N = pytest.importorskip("spg_gb300.native")
    obj = _scenes()[name].copy()
    dt = 1 / 60
    if method == IR.SYMPLECTIC_EULER:
        dt = 1e-4   # explicit: below the bar's stability limit; start stretched by 2 % along x
        obj.x = obj.x0 + 0.02 * (obj.x0 - obj.x0.mean(0)) * np.array([1.0, 0.0, 0.0])
    gpu = N.ImplicitSolver([obj], dt=dt, substeps=1, gravity=scenes.GRAVITY, method=method)
    ref = IR.ImplicitSolver(obj, dt, 1, scenes.GRAVITY, method)
    failed = 0
    for _ in range(10):
        st = gpu.step()
        ref.step()
        failed += int(st.skipped_solves)
    xg, vg = gpu.state(0)
    xr, vr = ref.state()
    extent = float(np.ptp(obj.x0, axis=0).max())
    err = float(np.abs(xg - xr).max())
    moved = float(np.abs(xr - obj.x).max())
    print(f"method {method} on {name}: max |dx| {err:.3g} m after 10 steps (moved {moved:.3g} m), "
          f"failed substeps GPU/oracle {failed}/{ref.failed_substeps}")
    assert err <= 1e-4 * extent and err <= 1e-3 * moved
    if method in (IR.NEWTON_ROBUST, IR.QUASI_STATIC_NEWTON_ROBUST):
        assert failed == ref.failed_substeps
        assert gpu.step_size() == ref.current_dt


@pytest.mark.gpu
@pytest.mark.parametrize("method,name", [(IR.NEWTON_ROBUST, "stvk_cloth"), (IR.BDF2, "snh_beam")])
def test_changing_dt_between_steps_keeps_history(method, name):
    """setDt between steps: the robust step control and BDF2's previous state carry over
    (implicitEulerNewtonRobust.cpp:37-40 clamps m_currentDt to the new maximum; bdf2.cpp:66-67
    keeps m_xMinusOne / m_vMinusOne). Halving dt after five steps must match the oracle doing the same."""
    N = pytest.importorskip("spg_gb300.native")
    obj = _scenes()[name].copy()
    gpu = N.ImplicitSolver([obj], dt=1 / 60, substeps=1, gravity=scenes.GRAVITY, method=method)
    ref = IR.ImplicitSolver(obj, 1 / 60, 1, scenes.GRAVITY, method)
    for k in range(10):
        if k == 5:
            gpu.set_params(dt=1 / 120)
            ref.dt = 1 / 120
        gpu.step()
        ref.step()
    xg, _ = gpu.state(0)
    xr, _ = ref.state()
    err = float(np.abs(xg - xr).max())
    moved = float(np.abs(xr - obj.x).max())
    assert err <= 1e-4 * float(np.ptp(obj.x0, axis=0).max()) and err <= 1e-3 * moved
    if method == IR.NEWTON_ROBUST:
        assert gpu.step_size() == ref.current_dt
    p = N.ImplicitParams()
    C.memmove(C.byref(p), C.byref(gpu.params), C.sizeof(p))
    p.method = IR.NEWTON_DX
    assert N.STATUS[N.lib().spgx_implicit_set_params(gpu.h, C.byref(p))] == "INVALID_ARG"


@pytest.mark.gpu
@pytest.mark.parametrize("method", range(9))
def test_cpp_drop_in_matches_the_handle(method):
    """spg::solver::GpuImplicit (the BaseSolver drop-in for the reference's global solver
    classes) steps like the C ABI handle it wraps. Assembly sums element gradients and Hessian
    blocks with FP64 atomics, so two runs agree to rounding, not bit for bit."""
    N = pytest.importorskip("spg_gb300.native")
    from spg_gb300 import scenes as S
    scene = S.tet_beam(7, 3, 3)
    dt = 1e-4 if method == IR.SYMPLECTIC_EULER else 1 / 60
    x_cpp = scene.run_gpu_implicit(4, dt, 1, scenes.GRAVITY, method)
    h = N.ImplicitSolver(scene.objects, dt=dt, substeps=1, gravity=scenes.GRAVITY, method=method)
    for _ in range(4):
        h.step()
    np.testing.assert_allclose(x_cpp, h.state(0)[0], rtol=0, atol=1e-10)
