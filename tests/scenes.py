"""Benchmark scene definitions shared by the tests (built with the oracle's builders, which
restate the reference's apps/solverCompare.cpp scene code)."""
from __future__ import annotations

from oracle import pyoracle as O

GRAVITY = (0.0, 0.0, -9.81)


def stvk_from_lame(mu: float, lam: float):
    """(young, poisson) such that the reference's plane-stress StVK matrix has
    c11 = 2 mu + lambda, c12 = lambda, c33 = mu (membraneStvkEnergy.cpp:35-38)."""
    nu = lam / (2 * mu + lam)
    return (2 * mu + lam) * (1 - nu * nu), nu


def cloth_cfg1(rows=33):
    """1 m square, StVK mu = lambda = 1e4 N/m, bending 1e-3, 0.1 kg/m^2, two top corners
    pinned (anchor k 1e5 as the reference cloth), flat rest state."""
    young, nu = stvk_from_lame(1e4, 1e4)
    return O.build_cloth(0.1, 1.0, 1.0, rows, rows, young, nu, 1e-3, 1e5, True)


def beam_cfg2(nx=41, ny=11, nz=11):
    """SNH bar of 2.5 cm cells split in 6 tets, E 1e6, nu 0.45, 1000 kg/m^3, x-min face
    anchored with the reference beam's anchor stiffness 1e4."""
    sx, sy, sz = 0.025 * (nx - 1), 0.025 * (ny - 1), 0.025 * (nz - 1)
    return O.build_tet_beam(1000.0 * sx * sy * sz, sx, sy, sz, nx, ny, nz, 1e6, 0.45, 1e4, 6)


def spring_cloth_cfg3(n=513, seed=12345):
    """Spring cloth with the large-cloth spacing (2 m at 513 vertices per side): springs
    k 1e4 on all edges, bending 1e-4, 0.1 kg/m^2, in-plane rest jitter N(0, (0.1 edge)^2),
    top row anchored (k 1e5)."""
    w = 2.0 * (n - 1) / 512
    return O.build_spring_cloth(0.1 * w * w, w, w, n, n, 1e4, 1e-4, 1e5, 0.1, seed)


def patch_batch_cfg4(n_patches=512, n_min=16, n_max=128, seed=2024):
    """Independent 1 m StVK patches (mu, lambda ~ logU[1e3, 1e5], bending ~ logU[1e-5, 1e-2],
    one random corner anchored)."""
    return O.build_patch_batch(n_patches, n_min, n_max, 1e3, 1e5, 1e-5, 1e-2, 0.1, 1e5, seed)


# ---------------------------------------------------------------------------------------
# Scenes with the energy types 6-14. Their per-stencil data restate the reference's
# addStencil() + preparePrecomputations() (test infrastructure, numpy).

import numpy as np  # noqa: E402


def _lame(young, poisson):
    mu = young / (2 * (1 + poisson))
    lam = young * poisson / ((1 + poisson) * (1 - 2 * poisson)) + 1e-20
    return lam, mu


def tet_params(x0, tets, young, poisson):
    """StvkEnergy / StableSquaredNeoHookeanEnergy (stvkEnergy.cpp:61-108,
    stableSquaredNeoHookeanEnergy.cpp:33-75): [Dinv (3x3 row-major), lambda V, mu V,
    1/(lambda V), 1/(mu V)]."""
    lam, mu = _lame(young, poisson)
    out = []
    for t in tets:
        Dm = np.column_stack([x0[t[1]] - x0[t[0]], x0[t[2]] - x0[t[0]], x0[t[3]] - x0[t[0]]])
        V = np.linalg.det(Dm) / 6.0
        assert V > 0
        out.append(np.concatenate([np.linalg.inv(Dm).reshape(-1), [lam * V, mu * V, 1 / (lam * V), 1 / (mu * V)]]))
    return np.array(out)


def membrane_params(x0, tris, k):
    """MembraneBaraffWitkinEnergy / MembraneChoiEnergy (membraneBaraffWitkinEnergy.cpp:42-70,
    membraneChoiEnergy.cpp:45-73): [Dinv (2x2 row-major) of the z = 0 rest triangle,
    k_i * area, 1 / (k_i * area)]."""
    k = np.asarray(k, dtype=np.float64)
    out = []
    for t in tris:
        assert np.all(x0[t][:, 2] == 0.0)
        u = (x0[t[1]] - x0[t[0]])[:2]
        v = (x0[t[2]] - x0[t[0]])[:2]
        Dm = np.column_stack([u, v])
        A = 0.5 * (u[0] * v[1] - v[0] * u[1])
        assert A > 0
        out.append(np.concatenate([np.linalg.inv(Dm).reshape(-1), k * A, 1 / (k * A)]))
    return np.array(out)


def bw_bending_params(x0, stencils, k):
    """BaraffWitkinBendingEnergy (baraffWitkinBendingEnergy.cpp:40-76): [restTheta, k, 1/k]."""
    out = []
    for s in stencils:
        e0 = x0[s[1]] - x0[s[0]]
        e3 = x0[s[2]] - x0[s[1]]
        e4 = x0[s[3]] - x0[s[1]]
        n1 = np.cross(e0, e3)
        n1 /= np.linalg.norm(n1)
        n2 = -np.cross(e0, e4)
        n2 /= np.linalg.norm(n2)
        th = np.arctan2(np.dot(np.cross(n1, n2), e0 / np.linalg.norm(e0)), np.dot(n1, n2))
        out.append([th, k, 1 / k])
    return np.array(out)


def quad_bending_params(x0, stencils, k):
    """QuadraticBendingEnergy (quadraticBendingEnergy.cpp:48-93): the cotangent weights
    [c0, c1, c2, c3] of the Laplacian, k * 3 / (area of the two triangles), its inverse."""
    def cot(a, b):
        return np.dot(a, b) / np.linalg.norm(np.cross(a, b))
    out = []
    for s in stencils:
        x = x0[s]
        e0, e1, e2 = x[1] - x[0], x[2] - x[0], x[3] - x[0]
        e3, e4 = x[2] - x[1], x[3] - x[1]
        c01, c02, c03, c04 = cot(e0, e1), cot(e0, e2), cot(-e0, e3), cot(-e0, e4)
        keff = k * 3 / (0.5 * (np.linalg.norm(np.cross(e0, e1)) + np.linalg.norm(np.cross(e0, e2))))
        out.append([c03 + c04, c01 + c02, -c01 - c03, -c02 - c04, keff, 1 / keff])
    return np.array(out)


def continuum_spring_params(x0, pairs, k):
    """SpringContinuumEnergy / SpringSquaredContinuumEnergy (springContinuumEnergy.cpp:19-34):
    [L0, k L0, 1 / (k L0)]."""
    L0 = np.linalg.norm(x0[pairs[:, 0]] - x0[pairs[:, 1]], axis=1)
    return np.column_stack([L0, k * L0, 1 / (k * L0)])


def _energy(etype, stencils, params):
    return O.Energy(etype, np.ascontiguousarray(stencils, dtype=np.int32), np.ascontiguousarray(params))


def beam_tet_variant(etype, nx=9, ny=4, nz=4, young=1e6, poisson=0.45, load=False):
    """The SNH bar's tets and anchors with StVK tet (6) or stable squared neo-Hookean (7)
    elasticity in place of SNH; with load, a static load (14) pulls the free end's vertices
    down and sideways with twice their weight."""
    b = beam_cfg2(nx, ny, nz)
    tets = next(e for e in b.energies if e.type == O.SNH).stencils
    energies = [_energy(etype, tets, tet_params(b.x0, tets, young, poisson))]
    energies += [e for e in b.energies if e.type == O.ANCHOR]
    if load:
        end = np.flatnonzero(b.x0[:, 0] >= b.x0[:, 0].max() - 1e-12).astype(np.int32).reshape(-1, 1)
        d = np.array([0.0, 0.6, -0.8])
        k = 2 * 9.81 * b.mass[end[:, 0]]
        energies.append(_energy(O.STATIC_LOAD, end, np.column_stack([k, np.tile(d, (len(k), 1))])))
    return O.SceneObject(b.x.copy(), b.mass.copy(), energies, None, b.x0.copy())


def cloth_variant(kind, rows=9):
    """The StVK cloth's triangles and bending stencils with Baraff-Witkin (8) or Choi (9)
    membranes and Baraff-Witkin (10) or quadratic (11) bending, plus its anchors."""
    c = cloth_cfg1(rows)
    tris = next(e for e in c.energies if e.type == O.STVK).stencils
    bend = next(e for e in c.energies if e.type == O.BENDING).stencils
    membrane, bending = kind
    k = [1e3, 1e3, 5e2] + ([5e2] if membrane == O.CHOI_MEMBRANE else [])
    energies = [_energy(membrane, tris, membrane_params(c.x0, tris, k))]
    if bending == O.BW_BENDING:
        energies.append(_energy(bending, bend, bw_bending_params(c.x0, bend, 1e-3)))
    else:
        energies.append(_energy(bending, bend, quad_bending_params(c.x0, bend, 1e-3)))
    energies += [e for e in c.energies if e.type == O.ANCHOR]
    return O.SceneObject(c.x.copy(), c.mass.copy(), energies, None, c.x0.copy())


def spring_variant(n=9, load=False):
    """The spring cloth's edges as continuum springs (12) and squared continuum springs (13)
    whose small-strain stiffnesses (k / L0 and 4 k / L0) are each about half the spring
    cloth's 1e4 N/m, and its anchors; with load, a static load (14) about the vertex weight on
    the bottom row. (A point load on a flat cloth makes its out-of-plane response nearly
    singular: trajectories then depend chaotically on rounding, so parity runs use the load on
    the tet bar instead.)"""
    s = spring_cloth_cfg3(n)
    pairs = next(e for e in s.energies if e.type == O.SPRING).stencils
    energies = [_energy(O.SPRING_CONT, pairs, continuum_spring_params(s.x0, pairs, 20.0)),
                _energy(O.SPRING_SQ_CONT, pairs, continuum_spring_params(s.x0, pairs, 5.0))]
    energies += [e for e in s.energies if e.type == O.ANCHOR]
    if load:
        bottom = np.arange((n - 1) * n, n * n, dtype=np.int32).reshape(-1, 1)
        d = np.array([0.0, 0.6, 0.8])
        weight = float(s.mass.max()) * 9.81
        energies.append(_energy(O.STATIC_LOAD, bottom, np.tile(np.concatenate([[weight], d]), (n, 1))))
    return O.SceneObject(s.x.copy(), s.mass.copy(), energies, None, s.x0.copy())


def truss_variant(nx=5, ny=3, nz=3, k_cont=2e3, k_sq=5e2):
    """The SNH bar's tet edges as continuum springs (12) and squared continuum springs (13),
    with its anchors: a 3D truss, well conditioned for implicit solves (a flat cloth at rest has
    no transverse stiffness)."""
    b = beam_cfg2(nx, ny, nz)
    tets = next(e for e in b.energies if e.type == O.SNH).stencils
    pairs = set()
    for t in tets:
        for i in range(4):
            for j in range(i + 1, 4):
                pairs.add((min(t[i], t[j]), max(t[i], t[j])))
    pairs = np.array(sorted(pairs), dtype=np.int32)
    energies = [_energy(O.SPRING_CONT, pairs, continuum_spring_params(b.x0, pairs, k_cont)),
                _energy(O.SPRING_SQ_CONT, pairs, continuum_spring_params(b.x0, pairs, k_sq))]
    energies += [e for e in b.energies if e.type == O.ANCHOR]
    return O.SceneObject(b.x.copy(), b.mass.copy(), energies, None, b.x0.copy())

