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
tolerance (from the extrapolated guess, which converges in a few hundred iterations), and
(features at the step's start, (x* - y) / l at its end) is recorded for a random subset of
the vertices. The network learns the remainder (x* - x_e) / l of the extrapolated guess x_e.

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


def extrapolation_offset(features: np.ndarray) -> np.ndarray:
    """(x_e - y) / l of the extrapolated guess from recorded features: d1 - d2 - h^2 g over l."""
    return features[:, 3:6] - features[:, 6:9] - features[:, 15:18]


def generate(episodes=16, steps=60, vertices_per_episode=270_000, sizes=(65, 129), keep=1 / 16, tol=1e-5,
             max_iterations=3000, max_speed=30.0, seed=7, device=0, time_budget=None, log=print):
    """Runs the episodes on the GPU solver (each step solved to the tolerance, starting from
    the extrapolated guess) and returns (features [m x 24], network targets [m x 3]): the
    recorded (x* - y) / l minus the extrapolated guess's offset.

    A patch whose speed exceeds max_speed is folding without self-contact handling (the
    reference's VBD has none either) and would stall the shared tolerance test: it is put
    back at rest in its initial pose and its rows are left out. A reset restarts the
    displacement history of the whole scene, so the step after it is not recorded; neither
    is a step that did not reach the tolerance (its target would not be a solution)."""
    rng = np.random.default_rng(seed)
    feats, targs = [], []
    t0 = time.time()
    for ep in range(episodes):
        if time_budget is not None and time.time() - t0 > time_budget:
            log(f"generation time budget reached after {ep} episodes")
            break
        n = int(sizes[ep % len(sizes)])
        count = max(1, vertices_per_episode // (n * n))
        patches = [random_patch(n, rng) for _ in range(count)]
        g = random_gravity(rng)
        solver = N.VbdSolver(patches, dt=DT, iterations=20, gravity=g, tolerance=tol, max_iterations=max_iterations,
                             check_interval=50, device=device)
        solver.set_warm_start(None, mode=2)
        patch_of_row = solver.vertex_order() // (n * n)
        bad = np.zeros(count, bool)
        ep_f, ep_t, ep_p, its, unconverged, skip = [], [], [], [], 0, False
        for k in range(steps):
            st, f, t = solver.step_record()
            its.append(int(st.iterations))
            unconverged += int(not st.converged)
            speed = np.zeros(count)
            v = np.linalg.norm(f[:, 3:6], axis=1) * (DT * G0)
            np.maximum.at(speed, patch_of_row, np.where(np.isfinite(v), v, np.inf))
            if not skip and st.converged:
                sel = rng.random(f.shape[0]) < keep
                ep_f.append(f[sel])
                ep_t.append(t[sel] - extrapolation_offset(f[sel]))
                ep_p.append(patch_of_row[sel])
            skip = False
            fresh = np.flatnonzero((speed > max_speed) & ~bad)
            if fresh.size:
                bad[fresh] = True
                for p in fresh:
                    solver.set_state(int(p), patches[p].x, np.zeros_like(patches[p].x))
                skip = True
        solver.close()
        if ep_p:
            rows = ~bad[np.concatenate(ep_p)]
            feats.append(np.concatenate(ep_f)[rows])
            targs.append(np.concatenate(ep_t)[rows])
        log(f"episode {ep}: {count} patches of {n}^2 ({int(bad.sum())} folded, dropped), gravity "
            f"{np.round(g, 2).tolist()}, iterations/step mean {np.mean(its):.0f} max {max(its)}, "
            f"{unconverged} steps unconverged, {time.time() - t0:.0f} s")
    return np.concatenate(feats), np.concatenate(targs)


def output_scale(Y) -> float:
    """RMS of the corrections, the network's output unit (rows beyond 100 l are outliers)."""
    a = np.abs(Y).max(axis=1)
    return float(np.sqrt(np.mean(Y[a < 100.0] ** 2))) or 1.0


def fold_output_scale(w: np.ndarray, scale: float) -> np.ndarray:
    """Scales the last (linear) layer so the network outputs `scale` times its trained output."""
    w = w.copy()
    n_in, n_hid, n_out = 24, 128, 3
    off_w4 = n_in * n_hid + n_hid + 2 * (n_hid * n_hid + n_hid)
    w[off_w4:] *= scale  # W4 (128 x 3) and b4 (3)
    assert w.size == off_w4 + n_hid * n_out + n_out
    return w


def train(X, Y, stages=((12000, 1e-3), (8000, 3e-4), (6000, 1e-4)), batch=4096, seed=11, device=0, log=print):
    """Trains a fresh network on (X, Y / scale) with the library's Adam and folds the scale into
    its last layer; returns (mlp, history, scale)."""
    scale = output_scale(Y)
    keep = np.abs(Y).max(axis=1) < 100.0
    Xt, Yt = X[keep], (Y[keep] / scale).astype(np.float32)
    mlp = N.Mlp(seed=seed, device=device)
    hist = []
    for i, (steps, lr) in enumerate(stages):
        t0 = time.time()
        loss = mlp.train(Xt, Yt, steps=steps, batch=batch, lr=lr, seed=seed + 100 * i)
        hist.append({"steps": steps, "lr": lr, "last_batch_loss": float(loss), "seconds": time.time() - t0})
        log(f"stage {i}: {steps} steps at lr {lr}: last minibatch loss {loss:.4g} ({time.time() - t0:.1f} s)")
    mlp.set_weights(fold_output_scale(mlp.weights(), scale))
    return mlp, hist, scale


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--episodes", type=int, default=16)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--keep", type=float, default=1 / 16)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--max-iterations", type=int, default=3000)
    ap.add_argument("--time-budget", type=float, default=600.0, help="seconds of data generation at most")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--sizes", type=int, nargs="+", default=[65, 129],
                    help="patch side lengths (vertices), one per episode in turn")
    args = ap.parse_args(argv)
    os.makedirs(args.out, exist_ok=True)
    t0 = time.time()
    X, Y = generate(episodes=args.episodes, steps=args.steps, keep=args.keep, tol=args.tol,
                    max_iterations=args.max_iterations, device=args.device, time_budget=args.time_budget,
                    sizes=tuple(args.sizes))
    t_gen = time.time() - t0
    print(f"{X.shape[0]} rows in {t_gen:.0f} s; target rms {np.sqrt(np.mean(Y ** 2)):.4g}", flush=True)
    # Held-out rows (the last 2 %) measure the fit.
    m = X.shape[0]
    cut = int(m * 0.98)
    mlp, hist, scale = train(X[:cut], Y[:cut], device=args.device)
    pred = mlp.forward(X[cut:])
    mse = float(np.mean((pred - Y[cut:]) ** 2))
    base = float(np.mean(Y[cut:] ** 2))
    w = mlp.weights()
    np.save(os.path.join(args.out, "warm_start_spring_cloth.npy"), w)
    meta = {"rows": int(m), "episodes": args.episodes, "sizes": list(args.sizes), "steps_per_episode": args.steps,
            "row_fraction": args.keep,
            "tolerance": args.tol, "max_iterations": args.max_iterations, "generation_s": t_gen, "stages": hist,
            "output_scale": scale, "heldout_mse": mse, "heldout_mse_of_zero_guess": base,
            "params": int(w.size)}
    with open(os.path.join(args.out, "warm_start_spring_cloth.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta), flush=True)


if __name__ == "__main__":
    main()
