"""Runs independent FP64 oracle VBD solves in parallel worker processes (test infrastructure).

Small objects leave the oracle's per-colour OpenMP loops mostly idle, so many of them are
solved one per process instead, each process single-threaded. The pool is started with
`spawn`: a forked child of a process that has already used CUDA can hang.
"""
from __future__ import annotations

import multiprocessing as mp
import os
from concurrent.futures import ProcessPoolExecutor


def _run(obj, dt, iterations, steps, gravity):
    from oracle import pyoracle as O
    r = O.Vbd(obj, dt, 1, iterations, gravity, O.VERTEX_AD)
    for _ in range(steps):
        r.step()
    return r.state()[0]


def _solve(args):
    obj, dt, iterations, steps, gravity, perturb = args
    import numpy as np
    from oracle import pyoracle as O
    O.set_threads(1)
    x = _run(obj, dt, iterations, steps, gravity)
    if not perturb:
        return x, None
    # The same solve from start positions moved by perturb (seeded per object size): how far
    # the FP64 trajectory itself moves measures how much rounding it amplifies.
    p = obj.copy()
    p.x = p.x + np.random.default_rng(obj.nv).normal(scale=perturb, size=p.x.shape)
    return x, float(np.abs(_run(p, dt, iterations, steps, gravity) - x).max())


def solve_many(objs, dt, iterations, steps, gravity, perturb=0.0, workers=None):
    """For each object, its positions after `steps` oracle VBD steps (one substep each) and,
    with perturb > 0, the largest change of those positions when the start positions are
    moved by N(0, perturb^2) (else None)."""
    workers = workers or max(1, min(len(objs), os.cpu_count() or 1))
    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_solve, [(o, dt, iterations, steps, gravity, perturb) for o in objs]))
