"""Learned warm start of GpuVBD: training data generated by the GPU solver itself, training with
the library's own MLP kernels, and the network shipped with the package.

The reference's VBD starts every step from the inertial guess y (spg/source/sim/solver/vbd.cpp:
78-83). The learned guess replaces y by y + l * MLP(features) when that lowers the residual;
the solver then iterates to the same tolerance as without it. Features, target and units are
defined in include/spgx.h (spgx_vbd_set_warm_start).

Training data: episodes of spring-cloth patches with the large cloth's material and spacing
(springs k = 1e4 on every edge of a 3.906 mm grid, bending 1e-4, 0.1 kg/m^2, in-plane rest
jitter), each patch rotated uniformly at random and pinned by a random pin set, under a
gravity direction drawn uniformly on the sphere per episode. Every step is solved to the
tolerance, and (features at the step's start, (x* - y) / l at its end) is recorded for a
random subset of the vertices.

Command line (on a GPU):  python -m spg_gb300.warm_start --out DIR [--episodes 30 ...]
writes DIR/warm_start_spring_cloth.npy (flat FP32 weights) and DIR/warm_start_spring_cloth.json.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from spg_gb300 import native as N
from spg_gb300 import scenes as S

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
WEIGHTS = os.path.join(WEIGHTS_DIR, "warm_start_spring_cloth.npy")
DT = 1.0 / 120.0
G0 = 9.81


def load_mlp(device=0, path=WEIGHTS) -> N.Mlp:
    """The shipped network (raises if the weights file is missing)."""
    w = np.load(path)
    return N.Mlp(seed=0, device=device, weights=w)


def random_rotation(rng) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def random_pins(n: int, rng) -> np.ndarray:
    """Vertex ids (row-major n x n grid) of a random pin set: one full edge, the two corners
    of an edge, one corner, a few vertices of an edge, or the centre vertex."""
    edge_ids = {0: np.arange(n), 1: np.arange(n) * n + n - 1, 2: (n - 1) * n + np.arange(n), 3: np.arange(n) * n}
    e = edge_ids[int(rng.integers(4))]
    kind = int(rng.integers(5))
    if kind == 0:
        return e
    if kind == 1:
        return np.array([e[0], e[-1]])
    if kind == 2:
        return np.array([e[0] if rng.random() < 0.5 else e[-1]])
    if kind == 3:
        return np.sort(rng.choice(e, size=min(n, int(rng.integers(2, 9))), replace=False))
    return np.array([(n // 2) * n + n // 2])


def random_patch(n: int, rng) -> S.SceneObject:
    """An n x n spring-cloth patch with the large cloth's spacing and material, rotated
    uniformly at random, pinned by a random pin set (anchor stiffness 1e5)."""
    obj = S.spring_cloth(n, seed=int(rng.integers(1, 2 ** 62))).objects[0]
    R = random_rotation(rng)
    c = obj.x.mean(0)
    x = (obj.x - c) @ R.T
    energies = []
    for e in obj.energies:
        if e.type == N.ANCHOR:
            pins = random_pins(n, rng)
            k, cmp = e.params[0, 3], e.params[0, 4]
            params = np.column_stack([x[pins], np.full(len(pins), k), np.full(len(pins), cmp)])
            energies.append(S.Energy(N.ANCHOR, pins.reshape(-1, 1).astype(np.int32), params))
        else:
            energies.append(e)
    return S.SceneObject(x=x, mass=obj.mass.copy(), energies=energies, v=np.zeros_like(x), x0=x.copy())


def random_gravity(rng) -> tuple:
    u = rng.standard_normal(3)
    u /= np.linalg.norm(u)
    return tuple(float(a) for a in G0 * u)


def generate(episodes=30, steps=60, vertices_per_episode=270_000, sizes=(33, 65, 129), keep=1 / 32, tol=1e-5,
             max_iterations=3000, seed=7, device=0, log=print):
    """Runs the episodes on the GPU solver and returns (features [m x 24], targets [m x 3])."""
    rng = np.random.default_rng(seed)
    feats, targs = [], []
    t0 = time.time()
    for ep in range(episodes):
        n = int(sizes[ep % len(sizes)])
        count = max(1, vertices_per_episode // (n * n))
        patches = [random_patch(n, rng) for _ in range(count)]
        g = random_gravity(rng)
        solver = N.VbdSolver(patches, dt=DT, iterations=20, gravity=g, tolerance=tol, max_iterations=max_iterations,
                             check_interval=100, device=device)
        solver.set_warm_start(None, enable=False)
        its = []
        for k in range(steps):
            st, f, t = solver.step_record()
            its.append(int(st.iterations))
            m = f.shape[0]
            sel = rng.random(m) < keep
            feats.append(f[sel])
            targs.append(t[sel])
        solver.close()
        log(f"episode {ep}: {count} patches of {n}^2, gravity {np.round(g, 2).tolist()}, iterations/step "
            f"mean {np.mean(its):.0f} max {max(its)}, {time.time() - t0:.0f} s")
    return np.concatenate(feats), np.concatenate(targs)


def train(X, Y, stages=((12000, 1e-3), (8000, 3e-4), (6000, 1e-4)), batch=4096, seed=11, device=0, log=print):
    """Trains a fresh network on (X, Y) with the library's Adam; returns (mlp, history)."""
    mlp = N.Mlp(seed=seed, device=device)
    hist = []
    for i, (steps, lr) in enumerate(stages):
        t0 = time.time()
        loss = mlp.train(X, Y, steps=steps, batch=batch, lr=lr, seed=seed + 100 * i)
        hist.append({"steps": steps, "lr": lr, "last_batch_loss": float(loss), "seconds": time.time() - t0})
        log(f"stage {i}: {steps} steps at lr {lr}: last minibatch loss {loss:.4g} ({time.time() - t0:.1f} s)")
    return mlp, hist


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--episodes", type=int, default=30)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--keep", type=float, default=1 / 32)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--max-iterations", type=int, default=3000)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    os.makedirs(args.out, exist_ok=True)
    t0 = time.time()
    X, Y = generate(episodes=args.episodes, steps=args.steps, keep=args.keep, tol=args.tol,
                    max_iterations=args.max_iterations, device=args.device)
    t_gen = time.time() - t0
    print(f"{X.shape[0]} rows in {t_gen:.0f} s; target rms {np.sqrt(np.mean(Y ** 2)):.4g}", flush=True)
    # Held-out rows (the last 2 %) measure the fit.
    m = X.shape[0]
    cut = int(m * 0.98)
    mlp, hist = train(X[:cut], Y[:cut], device=args.device)
    pred = mlp.forward(X[cut:])
    mse = float(np.mean((pred - Y[cut:]) ** 2))
    base = float(np.mean(Y[cut:] ** 2))
    w = mlp.weights()
    np.save(os.path.join(args.out, "warm_start_spring_cloth.npy"), w)
    meta = {"rows": int(m), "episodes": args.episodes, "steps_per_episode": args.steps, "row_fraction": args.keep,
            "tolerance": args.tol, "max_iterations": args.max_iterations, "generation_s": t_gen, "stages": hist,
            "heldout_mse": mse, "heldout_mse_of_zero_guess": base, "params": int(w.size)}
    with open(os.path.join(args.out, "warm_start_spring_cloth.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta), flush=True)


if __name__ == "__main__":
    main()
