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
