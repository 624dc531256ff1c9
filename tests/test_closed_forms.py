"""The closed forms behind the global solvers' spring and bending assembly (implicit.cu),
restated in numpy and checked against the oracle's full-element automatic differentiation.
- The dihedral gradient: dtheta/dx1 = (a.e) Na / (|e| |Na|^2) - (b.e) Nb / (|e| |Nb|^2),
  dtheta/dx2 = -|e| Na / |Na|^2, dtheta/dx3 = |e| Nb / |Nb|^2, dtheta/dx0 = -(their sum),
  with e = x1 - x0, a = x2 - x0, b = x3 - x0, Na = e x a, Nb = e x b. Times k C it must give
  the oracle's gradient of 1/2 k (theta - theta0)^2.
- The derivative of that gradient is the full Hessian: central differences of k C grad
  theta must give the oracle's 12 x 12 Hessian. The assembly takes that derivative by forward
  mode, one seeded vertex at a time.
- The spring's blocks: H_00 = H_11 = -H_01 = k((1 - L0/l) I + L0 d d^T / l^3)."""
import numpy as np

from oracle import pyoracle as O


def _theta_and_gradient(X):
    e, a, b = X[1] - X[0], X[2] - X[0], X[3] - X[0]
    Na, Nb = np.cross(e, a), np.cross(e, b)
    L = np.linalg.norm(e)
    ina, inb = 1.0 / Na.dot(Na), 1.0 / Nb.dot(Nb)
    g1 = (a.dot(e) / L) * ina * Na - (b.dot(e) / L) * inb * Nb
    g2 = -L * ina * Na
    g3 = L * inb * Nb
    theta = np.arctan2(-L * Na.dot(b), -Na.dot(Nb))
    return theta, np.stack([-(g1 + g2 + g3), g1, g2, g3])


def _random_hinges(n, seed):
    """Hinges near the cloth configuration (flaps on either side of the edge, bent by up to
    about 60 degrees), away from degenerate triangles."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        x0 = rng.normal(scale=0.1, size=3)
        e = np.array([1.0, 0.0, 0.0]) + rng.normal(scale=0.2, size=3)
        f2 = np.array([0.4, 0.8, 0.0]) + rng.normal(scale=0.2, size=3)
        f3 = np.array([0.6, -0.8, 0.0]) + rng.normal(scale=0.2, size=3)
        f3[2] += rng.uniform(-0.8, 0.8)
        out.append(np.stack([x0, x0 + e, x0 + f2, x0 + f3]) * rng.uniform(0.01, 2.0))
    return out


def test_dihedral_gradient_times_kc_is_the_oracle_gradient():
    for X in _random_hinges(200, 1):
        theta0, k = 0.1, 0.7
        theta, gt = _theta_and_gradient(X)
        g, _ = O.element_full(O.BENDING, X, np.array([theta0, k]))
        expect = k * (theta - theta0) * gt.reshape(-1)
        assert np.allclose(g, expect, rtol=1e-9, atol=1e-12 * np.abs(expect).max())


def test_derivative_of_the_closed_form_gradient_is_the_oracle_hessian():
    worst = 0.0
    for X in _random_hinges(60, 2):
        theta0, k = -0.2, 1.3
        _, H = O.element_full(O.BENDING, X, np.array([theta0, k]))
        h = 1e-6 * np.abs(X).max()
        J = np.zeros((12, 12))
        for c in range(12):
            Xp, Xm = X.copy(), X.copy()
            Xp.reshape(-1)[c] += h
            Xm.reshape(-1)[c] -= h
            tp, gp = _theta_and_gradient(Xp)
            tm, gm = _theta_and_gradient(Xm)
            J[:, c] = (k * (tp - theta0) * gp.reshape(-1) - k * (tm - theta0) * gm.reshape(-1)) / (2 * h)
        worst = max(worst, float(np.abs(J - H).max() / np.abs(H).max()))
    assert worst < 1e-5


def test_spring_blocks_are_the_oracle_hessian():
    rng = np.random.default_rng(3)
    for _ in range(50):
        X = rng.normal(size=(2, 3))
        L0, k = float(rng.uniform(0.2, 3.0)), float(rng.uniform(1.0, 1e4))
        g, H = O.element_full(O.SPRING, X, np.array([L0, k]))
        d = X[0] - X[1]
        l = np.linalg.norm(d)
        B = k * ((1 - L0 / l) * np.eye(3) + L0 * np.outer(d, d) / l ** 3)
        expect = np.block([[B, -B], [-B, B]])
        assert np.allclose(H, expect, rtol=1e-10, atol=1e-10 * np.abs(expect).max())
        s = k * (l - L0) / l
        assert np.allclose(g, np.concatenate([s * d, -s * d]), rtol=1e-10, atol=1e-12 * k)
