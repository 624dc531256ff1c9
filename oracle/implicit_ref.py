"""CPU oracle of the reference's global solvers (test infrastructure only; nothing in the
product imports it).

Restates, in FP64, the per-substep algorithms of spg/source/sim/solver/:
  implicitEulerNewtonDx.cpp:11-65, implicitEulerNewtonDv.cpp:11-68,
  implicitEulerNewtonRobust.cpp:11-138, implicitEulerBaraffWitkin.cpp:11-60, bdf2.cpp:11-83,
  staticNewton.cpp:11-52, quasiStaticNewton.cpp:11-56, quasiStaticNewtonRobust.cpp:11-151 and
  simplecticEuler.cpp:11-62,
with ImplicitEulerBase's system force, mass matrix, stiffness matrix and linear solve
(implicitEulerBase.cpp:102-240):
  f = M g - sum_e grad E_e(x); K = -sum_e hess E_e(x) (full element Hessians from the
  oracle's automatic differentiation, no definiteness projection); linear systems by
  Eigen::ConjugateGradient with the diagonal preconditioner and the stopping rule
  |r|^2 < tol^2 |b|^2 (tol 1e-5, 300 iterations, zero initial guess).
The robust variants keep their step size across steps (m_currentDt) and leave the objects at
the last line-search candidate, as the reference does.
"""
import numpy as np
import scipy.sparse as sp

from oracle import pyoracle as O

NEWTON_DX, NEWTON_DV, NEWTON_ROBUST, BARAFF_WITKIN, BDF2, STATIC_NEWTON, QUASI_STATIC_NEWTON, \
    QUASI_STATIC_NEWTON_ROBUST, SYMPLECTIC_EULER = range(9)


def conjugate_gradient(A, b, tol=1e-5, max_iterations=300):
    """Eigen::ConjugateGradient with DiagonalPreconditioner (the reference's solver)."""
    n = b.shape[0]
    x = np.zeros(n)
    rhs2 = float(b @ b)
    if rhs2 == 0.0:
        return x, 0, 0.0
    d = A.diagonal()
    inv = np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 1.0)
    thr = max(tol * tol * rhs2, np.finfo(float).tiny)
    r = b.copy()
    rr = float(r @ r)
    if rr < thr:
        return x, 0, np.sqrt(rr / rhs2)
    p = inv * r
    rz = float(r @ p)
    it = 0
    while it < max_iterations:
        Ap = A @ p
        alpha = rz / float(p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        rr = float(r @ r)
        it += 1
        if rr < thr:
            break
        z = inv * r
        rz_old, rz = rz, float(r @ z)
        p = z + (rz / rz_old) * p
    return x, it, np.sqrt(rr / rhs2)


class ImplicitSolver:
    """One of the reference's global solvers on one object. x, v are (V, 3) arrays."""

    def __init__(self, obj, dt, substeps, gravity, method=NEWTON_DX, cg_threshold=1e-5, cg_max_iterations=300):
        self.obj = obj.copy()
        self.method = method
        self.x = np.array(obj.x, dtype=np.float64)
        self.v = np.zeros_like(self.x) if obj.v is None else np.array(obj.v, dtype=np.float64)
        self.m = np.asarray(obj.mass, dtype=np.float64)
        self.M = np.repeat(self.m, 3)
        self.w = np.repeat(np.where(self.m == 0, 0.0, 1.0 / np.where(self.m == 0, 1.0, self.m)), 3)
        self.dt, self.substeps = dt, substeps
        self.g = np.asarray(gravity, dtype=np.float64)
        self.tol, self.max_it = cg_threshold, cg_max_iterations
        self.last_iterations = 0
        self.current_dt = -1.0
        self.successes = 0
        self.failed_substeps = 0
        self.xm1 = None
        self.vm1 = None

    # ImplicitEulerBase::getSystemForce / getSystemStiffnessMatrix (K = -H is returned as H)
    def _system(self, x, hessian=True, gravity=True):
        x = x.reshape(-1, 3)
        nv = x.shape[0]
        f = (self.m[:, None] * self.g[None, :]).reshape(-1) if gravity else np.zeros(3 * nv)
        rows, cols, vals = [], [], []
        for e in self.obj.energies:
            S = O.STENCIL_SIZE[e.type]
            for i in range(e.n):
                st = e.stencils[i]
                g, H = O.element_full(e.type, x[st], e.params[i])
                dof = (3 * st[:, None] + np.arange(3)[None, :]).reshape(-1)
                np.add.at(f, dof, -g)
                if hessian:
                    rows.append(np.repeat(dof, 3 * S))
                    cols.append(np.tile(dof, 3 * S))
                    vals.append(H.reshape(-1))
        if not hessian:
            return f
        n = 3 * nv
        if rows:
            H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
        else:
            H = sp.csr_matrix((n, n))
        return f, H

    def _solve(self, alpha, beta, H, b):
        """CG on alpha M + beta H (= alpha M - beta K)."""
        A = (sp.diags(alpha * self.M) + beta * H).tocsr()
        dx, it, _ = conjugate_gradient(A, b, self.tol, self.max_it)
        self._its += it
        return dx

    def step(self):
        self._its = 0
        x = self.x.reshape(-1).copy()
        v = self.v.reshape(-1).copy()
        m = self.method
        if m in (NEWTON_ROBUST, QUASI_STATIC_NEWTON_ROBUST):
            for _ in range(self.substeps):
                x, v = (self._newton_robust if m == NEWTON_ROBUST else self._quasi_static_robust)(x, v)
        else:
            h = self.dt / self.substeps
            for _ in range(self.substeps):
                x, v = self._substep(x, v, h)
        self.x, self.v = x.reshape(-1, 3), v.reshape(-1, 3)
        self.last_iterations = self._its

    def _substep(self, x, v, dt):
        m = self.method
        if m == NEWTON_DX:
            x0 = x.copy()
            x = x + v * dt
            f, H = self._system(x)
            invdt = 1.0 / dt
            dx = self._solve(invdt * invdt, 1.0, H, f)
            x = x + dx
            return x, (x - x0) * invdt
        if m == NEWTON_DV:
            x0, v0 = x.copy(), v.copy()
            x = x + v * dt
            f, H = self._system(x)
            dv = self._solve(1.0, dt * dt, H, dt * f)
            v = v0 + dv
            return x0 + v * dt, v
        if m == BARAFF_WITKIN:
            v0 = v.copy()
            f, H = self._system(x)
            dv = self._solve(1.0, dt * dt, H, dt * (f + dt * -(H @ v0)))
            v = v0 + dv
            return x + v * dt, v
        if m == BDF2:
            x0, v0 = x.copy(), v.copy()
            if self.xm1 is None:
                self.xm1, self.vm1 = x0.copy(), v0.copy()
            f, H = self._system(x)
            w = x0 - self.xm1 + 2 * dt * v0
            rhs = 1.0 / 3.0 * self.M * (v0 - self.vm1) + 2.0 / 3.0 * dt * (f + 1.0 / 3.0 * -(H @ w))
            dv = self._solve(1.0, 4.0 / 9.0 * (dt * dt), H, rhs)
            v = v0 + dv
            x = 4.0 / 3.0 * x0 - 1.0 / 3.0 * self.xm1 + 2.0 / 3.0 * v * dt
            self.xm1, self.vm1 = x0, v0
            return x, v
        if m == STATIC_NEWTON:
            f, H = self._system(x)
            return x + self._solve(0.0, -1.0, H, -f), v
        if m == QUASI_STATIC_NEWTON:
            f, H = self._system(x)
            dtdt = dt * dt
            return x + self._solve(1.0, dtdt, H, dtdt * f), v
        if m == SYMPLECTIC_EULER:
            v = v + np.tile(dt * self.g, x.size // 3)
            v = v + self.w * self._system(x, hessian=False, gravity=False) * dt
            return x + v * dt, v
        raise ValueError(m)

    def _current_step(self):
        max_dt = self.dt / self.substeps
        if self.current_dt == -1.0 or self.current_dt > max_dt:
            self.current_dt = max_dt
        return self.current_dt, max_dt

    def _after_substep(self, ok, max_dt):
        if not ok:
            self.current_dt *= 0.75
            self.successes = 0
            self.failed_substeps += 1
        else:
            self.successes += 1
            if self.successes > 5 and self.current_dt < max_dt:
                self.current_dt /= 0.75

    def _newton_robust(self, x, v, threshold=1e-5):
        dt, max_dt = self._current_step()
        ok = True
        x0, v0 = x.copy(), v.copy()
        it = 0
        x = x + v * dt
        vi = v0.copy()
        while True:
            f, H = self._system(x)
            rhs = dt * f - self.M * (vi - v0)
            r0 = float(np.linalg.norm(rhs))
            dv = self._solve(1.0, dt * dt, H, rhs)
            res, ls, alpha = r0, 0, 1.0
            while res >= r0 and ls < 5:
                v = vi + dv * alpha
                x = x0 + v * dt
                f = self._system(x, hessian=False)
                res = float(np.linalg.norm(dt * f - self.M * (v - v0)))
                if res < r0:
                    vi = v
                alpha *= 0.5
                ls += 1
            if res >= r0 and res > threshold:
                ok = False
            it += 1
            if not (res > threshold and ok and it < 5):
                break
        if res > threshold:
            ok = False
        if not ok:
            x, v = x0, v0
        self._after_substep(ok, max_dt)
        self.last_residual = res
        return x, v

    def _quasi_static_robust(self, x, v, threshold=1e-2):
        dt, max_dt = self._current_step()
        invdt = 1 / dt
        invdt2 = invdt * invdt
        ok = True
        x0 = x.copy()
        it = 0
        xi = x0.copy()
        while True:
            f, H = self._system(x)
            v = (x - x0) * invdt
            rhs = f - invdt * self.M * v
            r0 = float(np.linalg.norm(rhs))
            dx = self._solve(invdt2, 1.0, H, rhs)
            res, ls, alpha = r0, 0, 1.0
            while res >= r0 and ls < 5:
                x = xi + dx * alpha
                cand = x.copy()
                v = (x - x0) * invdt
                f = self._system(x, hessian=False)
                res = float(np.linalg.norm(f - invdt * self.M * v))
                if res < r0:
                    xi = cand
                alpha *= 0.5
                ls += 1
            if res >= r0 and res > threshold:
                ok = False
            it += 1
            if not (res > threshold and ok and it < 5):
                break
        if res > threshold:
            ok = False
        if not ok:
            x = x0
        self._after_substep(ok, max_dt)
        self.last_residual = res
        return x, v

    def state(self):
        return self.x.copy(), self.v.copy()


def ImplicitEuler(obj, dt, substeps, gravity, cg_threshold=1e-5, cg_max_iterations=300):
    """ImplicitEulerNewtonDx (the first solver restated here)."""
    return ImplicitSolver(obj, dt, substeps, gravity, NEWTON_DX, cg_threshold, cg_max_iterations)
