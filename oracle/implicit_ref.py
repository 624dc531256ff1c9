"""CPU oracle of the implicit Euler Newton step (test infrastructure only; nothing in the
product imports it).

Restates spg::solver::ImplicitEulerNewtonDx::step (spg/source/sim/solver/
implicitEulerNewtonDx.cpp:11-65) with ImplicitEulerBase::getSystemForce, getSystemMassMatrix,
getSystemStiffnessMatrix and solveLinearSystem (implicitEulerBase.cpp:102-240) in FP64:

  per substep: x0 = x; x = x + h v (integrateVelocities, particleGroup.cpp:57-63);
  f = M g - sum_e grad E_e(x); K = -sum_e hess E_e(x) (full element Hessians from the oracle's
  automatic differentiation, no definiteness projection);
  dx = CG(M / h^2 - K, f) with Eigen::ConjugateGradient's diagonal preconditioner and stopping
  rule |r|^2 < tol^2 |f|^2 (tol 1e-5, 300 iterations, zero initial guess);
  x = x + dx; v = (x - x0) / h.
"""
import numpy as np
import scipy.sparse as sp

from oracle import pyoracle as O


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


class ImplicitEuler:
    def __init__(self, obj, dt, substeps, gravity, cg_threshold=1e-5, cg_max_iterations=300):
        self.obj = obj.copy()
        self.x = np.array(obj.x, dtype=np.float64)
        self.v = np.zeros_like(self.x) if obj.v is None else np.array(obj.v, dtype=np.float64)
        self.m = np.asarray(obj.mass, dtype=np.float64)
        self.dt, self.substeps = dt, substeps
        self.g = np.asarray(gravity, dtype=np.float64)
        self.tol, self.max_it = cg_threshold, cg_max_iterations
        self.last_iterations = 0

    def _system(self, x):
        nv = x.shape[0]
        f = (self.m[:, None] * self.g[None, :]).reshape(-1)
        rows, cols, vals = [], [], []
        for e in self.obj.energies:
            S = O.STENCIL_SIZE[e.type]
            for i in range(e.n):
                st = e.stencils[i]
                g, H = O.element_full(e.type, x[st], e.params[i])
                dof = (3 * st[:, None] + np.arange(3)[None, :]).reshape(-1)
                np.add.at(f, dof, -g)
                rows.append(np.repeat(dof, 3 * S))
                cols.append(np.tile(dof, 3 * S))
                vals.append(H.reshape(-1))
        n = 3 * nv
        if rows:
            K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
        else:
            K = sp.csr_matrix((n, n))
        return f, K

    def step(self):
        h = self.dt / self.substeps
        its = 0
        for _ in range(self.substeps):
            x0 = self.x.copy()
            self.x = self.x + h * self.v
            f, H = self._system(self.x)
            A = sp.diags(np.repeat(self.m, 3) / (h * h)) + H
            dx, it, _ = conjugate_gradient(A.tocsr(), f, self.tol, self.max_it)
            its += it
            self.x = self.x + dx.reshape(-1, 3)
            self.v = (self.x - x0) / h
        self.last_iterations = its

    def state(self):
        return self.x.copy(), self.v.copy()
