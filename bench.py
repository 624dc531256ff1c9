#!/usr/bin/env python3
"""Benchmark of the GB300 VBD step on the large spring cloth (263,169 vertices).

One step = one spg::solver::VBD::step() equivalent on the 513x513 jittered spring cloth
(787,456 springs k = 1e4, 785,408 bending stencils k = 1e-4, row 0 anchored), 20 VBD
iterations per step at dt = 1/120 s, computed in FP32 on the GPU. Metric: vertex-solves/s =
vertices x iterations x steps / device time. Inputs are resident in HBM when the timed region
starts; L2 is flushed (256 MiB write) between timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference VBD (the oracle, reference-literal
full-element AD per incidence, OpenMP on all host cores) on bounded samples of the same
workload: the reference itself does not build here (its Eigen and TinyAD submodules are empty).
Multi-GPU runs are independent replicas (a single VBD mesh does not shard); value is the
aggregate over ranks with the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "VBD vertex-solves/s on 263k-vert cloth; time-to-residual 1e-5, warm vs plain"
UNIT = "vertex-solves/s"
ROWS = 513
IMPLICIT_PRECISION = ("FP64 state and assembly; CG in double-float (FP32 pairs, 48-bit significands) on the symmetric "
                      "matrix, one cooperative launch per solve (FP64 CG when the system leaves that range)")
ITERATIONS = 20
DT = 1.0 / 120.0
GRAVITY = (0.0, 0.0, -9.81)
WORKLOAD = ("spring cloth 513x513 over 2 m (263169 verts, 787456 springs k=1e4, 785408 bending k=1e-4, "
            "513 anchors), VBD 20 iterations/step, dt=1/120 s")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 0, 1
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return dist, rank, local, ws


def _device(local):
    return "cpu" if local is None else f"cuda:{local}"


def _barrier(dist, local):
    """Barrier across ranks (local is the CUDA device, or None for CPU/gloo ranks)."""
    if dist is None:
        return
    import torch
    if local is not None:
        torch.cuda.synchronize(local)
    dist.barrier()


def _max_over_ranks(dist, local, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=_device(local))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(dist, local, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=_device(local))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms while active."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes_per_iteration(obj) -> int:
    """Compulsory FP32 bytes of one VBD iteration: per vertex 48 B (x read, x write, y and
    mass), a 4 B incidence offset, 4 B per incidence, and every element record once (spring
    16 B, bending 24 B, StVK 40 B, SNH 64 B, anchor 20 B)."""
    from spg_gb300 import native as N
    rec = {N.SPRING: 16, N.BENDING: 24, N.STVK: 40, N.SNH: 64, N.ANCHOR: 20}
    nv = obj.nv
    n_inc = sum(e.stencils.size for e in obj.energies)
    return 48 * nv + 4 * (nv + 1) + 4 * n_inc + sum(rec[e.type] * e.n for e in obj.energies)


def xpbd_algorithmic_bytes_per_substep(obj) -> int:
    """Compulsory bytes of one XPBD substep (one projection sweep over every stencil) in the
    FP32 device layout: each stencil's record once (spring: indices, rest length, stiffness
    16 B + compliance 4 B; bending: indices 16 B + angle, stiffness, compliance 16 B; anchor:
    target and stiffness 16 B + compliance 8 B + vertex 4 B), and each vertex's state read and
    written once (base and delta 32 B each way, velocity 16 B each way, the substep-start delta
    and the inertial target 16 B each written, inverse mass 4 B read)."""
    rec = {1: 20, 2: 28, 3: 32}
    n = sum(rec.get(e.type, 0) * e.n for e in obj.energies)
    return int(n + obj.nv * (32 + 32 + 16 + 16 + 16 + 16 + 4))


def _measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic_per_iteration(kernel_name):
    """DRAM bytes per colour sweep of the given kernel from its committed ncu summary, when present."""
    p = os.path.join(ROOT, "profiles", f"{kernel_name}_spring_cloth_513.json")
    try:
        with open(p) as f:
            return float(json.load(f)["dram_bytes_per_sweep"])
    except (OSError, KeyError, ValueError):
        return None


def cpu_baseline(target_s: float = 12.0) -> dict:
    """The oracle (CPU restatement of the reference VBD, reference-literal full-element AD per
    incidence, OpenMP over each colour group) on whole colour sweeps of the same cloth, until
    about target_s seconds of sweeping have run."""
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    w = 2.0
    obj = O.build_spring_cloth(0.1 * w * w, w, w, ROWS, ROWS, 1e4, 1e-4, 1e5, 0.1, 12345)
    s = O.Vbd(obj, DT, 1, ITERATIONS, GRAVITY, O.FULL_AD)
    s.begin_substep()
    done = 0
    t0 = time.perf_counter()
    ncol = s.n_colors()
    c = 0
    while True:
        s.iterate_color(c % ncol)
        done += s.color_size(c % ncol)
        c += 1
        if time.perf_counter() - t0 >= target_s and c >= ncol:
            break
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{c} colour phases ({done} vertex-solves, {c / ncol:.2f} sweeps) of the 513x513 cloth, "
                      f"full-element FP64 AD per incidence, {dt:.1f} s"}


def time_to_residual(local, tol=1e-5, prefix=2, steps=3, max_iterations=60000, mode=0, mlp=None) -> dict:
    """Wall time of VBD steps run to ||M/h^2 (x - y) + grad E(x)|| <= tol ||grad E(y)|| (FP64-reduced
    residual, checked every 200 iterations, the last interval cut to what the observed decay rate
    needs) on the 513x513 cloth. A fresh solver starts from rest;
    the first `prefix` steps build the displacement history and are not timed; the next `steps`
    steps are timed with CUDA events on the solver's stream. mode: 0 inertial guess (the
    reference's), 1 learned (mlp), 2 extrapolated acceleration; used for every step of the run."""
    from spg_gb300 import native as N
    from spg_gb300 import scenes as S
    obj = S.spring_cloth(ROWS).objects[0]
    solver = N.VbdSolver([obj], dt=DT, iterations=ITERATIONS, gravity=GRAVITY, device=local,
                         tolerance=tol, max_iterations=max_iterations, check_interval=200)
    solver.set_warm_start(mlp, mode=mode)
    rows = []
    for k in range(prefix + steps):
        st = solver.step()
        if k >= prefix:
            rows.append({"iterations": int(st.iterations), "converged": bool(st.converged),
                         "device_ms": float(st.device_ms),
                         "relative_residual": st.residual_final / st.residual_initial,
                         "guess_accepted": int(st.warm_accepted),
                         "guess_relative_residual": (st.residual_warm / st.residual_initial) if mode else 1.0})
    solver.close()
    return {"ms_total": sum(r["device_ms"] for r in rows), "iterations_total": sum(r["iterations"] for r in rows),
            "steps": rows}


def time_to_residual_legs(local) -> dict:
    """Plain, extrapolated and learned initial guesses under the same protocol."""
    from spg_gb300 import warm_start as WS
    out = {"tolerance": 1e-5, "normaliser": "||grad E(y)|| at the inertial guess y",
           "protocol": "fresh solver from rest; 2 untimed steps, then 3 timed steps",
           "check_interval": "200 iterations, the last one cut to what the decay rate between the last two checks needs",
           "plain": time_to_residual(local, mode=0),
           "extrapolated": time_to_residual(local, mode=2)}
    if os.path.exists(WS.WEIGHTS):
        mlp = WS.load_mlp(local)
        out["learned"] = time_to_residual(local, mode=1, mlp=mlp)
        out["learned_speedup_over_plain"] = out["plain"]["ms_total"] / out["learned"]["ms_total"]
        out["learned_speedup_over_extrapolated"] = out["extrapolated"]["ms_total"] / out["learned"]["ms_total"]
        mlp.close()
    out["extrapolated_speedup_over_plain"] = out["plain"]["ms_total"] / out["extrapolated"]["ms_total"]
    # A compact summary as the last key: the end of the JSON line is what a truncated log keeps.
    summ = {}
    for leg in ("plain", "extrapolated", "learned"):
        if leg in out:
            summ[leg] = {"ms": round(out[leg]["ms_total"], 3), "iterations": out[leg]["iterations_total"],
                         "per_step_iterations": [r["iterations"] for r in out[leg]["steps"]],
                         "guess_accepted": [r["guess_accepted"] for r in out[leg]["steps"]],
                         "converged": all(r["converged"] for r in out[leg]["steps"])}
    summ["speedup_learned_over_plain"] = out.get("learned_speedup_over_plain")
    summ["speedup_learned_over_extrapolated"] = out.get("learned_speedup_over_extrapolated")
    summ["speedup_extrapolated_over_plain"] = out["extrapolated_speedup_over_plain"]
    out["summary"] = summ
    return out


def _timed_steps(solver, steps):
    for _ in range(3):
        solver.step()
    return [solver.step().device_ms for _ in range(steps)]


def other_configs(local, only=None) -> dict:
    """The other benchmark configurations, each timed with CUDA events on its solver's stream
    (vertex-solves/s = vertices x iterations / device time; XPBD in steps/s). With `only`,
    just the configuration of that name (a single case for profiling)."""
    from spg_gb300 import native as N
    from spg_gb300 import scenes as S

    def want(name):
        return only is None or only == name

    out = {}
    cloth = S.cloth(33).objects[0]
    beam = S.tet_beam().objects[0]
    big = S.spring_cloth(ROWS).objects[0] if (only is None or "513" in only) else None
    if want("cloth_33x33_stvk_100it"):
        s = N.VbdSolver([cloth], dt=1 / 60, iterations=100, gravity=GRAVITY, device=local)
        ms = statistics.mean(_timed_steps(s, 10))
        out["cloth_33x33_stvk_100it"] = {"vertex_solves_per_s": cloth.nv * 100 / (ms * 1e-3), "ms_per_step": ms,
                                         "launch": list(s.launch())}
        s.close()
    if want("snh_beam_41x11x11_50it"):
        s = N.VbdSolver([beam], dt=1 / 60, iterations=50, gravity=GRAVITY, device=local)
        ms = statistics.mean(_timed_steps(s, 10))
        out["snh_beam_41x11x11_50it"] = {"vertex_solves_per_s": beam.nv * 50 / (ms * 1e-3), "ms_per_step": ms,
                                         "launch": list(s.launch())}
        s.close()
    if want("batch_512_patches_30it"):
        batch = S.patch_batch(512, 16, 128, seed=2024).objects
        nv = sum(o.nv for o in batch)
        peak, peak_kind = _measured_peaks()
        alg = sum(algorithmic_bytes_per_iteration(o) for o in batch)

        def roofline(ms_step):
            achieved = alg * 30 / (ms_step * 1e-3) / 1e9
            return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "peak_source": peak_kind, "algorithmic_bytes_per_sweep": alg}

        s = N.VbdSolver(batch, dt=1 / 60, iterations=30, gravity=GRAVITY, device=local)
        ms = statistics.mean(_timed_steps(s, 5))
        entry = {"vertex_solves_per_s": nv * 30 / (ms * 1e-3), "ms_per_step": ms, "vertices": nv,
                 "colors": int(s.n_colors(-1)), "launch": list(s.launch()), "graph": True, "roofline": roofline(ms)}
        s.close()
        # The dataflow kernel on the same batch, beside the autotuner's pick.
        s = N.VbdSolver(batch, dt=1 / 60, iterations=30, gravity=GRAVITY, device=local, kernel=3)
        ms3 = statistics.mean(_timed_steps(s, 5))
        entry["dataflow_kernel"] = {"vertex_solves_per_s": nv * 30 / (ms3 * 1e-3), "ms_per_step": ms3,
                                    "launch": list(s.launch()), "roofline": roofline(ms3)}
        s.close()
        out["batch_512_patches_30it"] = entry
    if want("implicit_euler_cloth_33x33"):
        imp = N.ImplicitSolver([cloth], dt=1 / 60, substeps=1, gravity=GRAVITY, device=local)
        stats = [imp.step() for _ in range(8)][3:]
        out["implicit_euler_cloth_33x33"] = {"ms_per_step": statistics.mean(st.device_ms for st in stats),
                                             "cg_iterations": [int(st.iterations) for st in stats],
                                             "precision": IMPLICIT_PRECISION}
        imp.close()
    if want("implicit_euler_spring_cloth_513"):
        imp = N.ImplicitSolver([big], dt=DT, substeps=1, gravity=GRAVITY, device=local)
        stats = [imp.step() for _ in range(4)][1:]
        ms = statistics.mean(st.device_ms for st in stats)
        its = [int(st.iterations) for st in stats]
        # The same steps with no CG iteration give the assembly's share of the step.
        imp0 = N.ImplicitSolver([big], dt=DT, substeps=1, gravity=GRAVITY, device=local, cg_max_iterations=0)
        ms0 = statistics.mean(st.device_ms for st in [imp0.step() for _ in range(4)][1:])
        imp0.close()
        out["implicit_euler_spring_cloth_513"] = {"ms_per_step": ms,
                                                  "us_per_cg_iteration": (ms - ms0) * 1e3 / max(1, statistics.mean(its)),
                                                  "cg_iterations": its,
                                                  "converged": [bool(st.converged) for st in stats],
                                                  "precision": IMPLICIT_PRECISION}
        imp.close()
    if want("global_solvers_snh_beam_41x11x11"):
        names = ["newton_dx", "newton_dv", "newton_robust", "baraff_witkin", "bdf2", "static_newton",
                 "quasi_static_newton", "quasi_static_newton_robust", "symplectic_euler"]
        solvers = {}
        for method, name in enumerate(names):
            dt = 1e-4 if name == "symplectic_euler" else 1 / 60
            imp = N.ImplicitSolver([beam], dt=dt, substeps=1, gravity=GRAVITY, device=local, method=method)
            stats = [imp.step() for _ in range(5)][2:]
            solvers[name] = {"ms_per_step": statistics.mean(st.device_ms for st in stats),
                             "cg_iterations": [int(st.iterations) for st in stats]}
            imp.close()
        out["global_solvers_snh_beam_41x11x11"] = {"dt": "1/60 s (symplectic Euler 1e-4 s)", "precision": IMPLICIT_PRECISION,
                                                   "solvers": solvers}
    if want("xpbd_spring_cloth_513_20substeps"):
        peak, peak_kind = _measured_peaks()
        alg = xpbd_algorithmic_bytes_per_substep(big)
        entry = {}
        for kernel, name in ((3, "synchronised"), (2, "dataflow"), (1, "phase_launches")):
            x = N.XpbdSolver([big], dt=DT, substeps=20, gravity=GRAVITY, device=local, kernel=kernel)
            ms = statistics.mean(_timed_steps(x, 5))
            achieved = alg * 20 / (ms * 1e-3) / 1e9
            entry[name] = {"steps_per_s": 1e3 / ms, "ms_per_step": ms,
                           "vertex_substeps_per_s": big.nv * 20 / (ms * 1e-3),
                           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                        "frac": achieved / peak, "peak_source": peak_kind,
                                        "algorithmic_bytes_per_substep": alg}}
            x.close()
        out["xpbd_spring_cloth_513_20substeps"] = entry
    if want("mlp_inference_spring_cloth_513"):
        # The learned warm start's network on every vertex of the 513x513 cloth: host arrays in
        # and out through the C ABI (the kernel's own time is in the ncu launch list).
        from spg_gb300 import warm_start as WS
        rng = np.random.default_rng(0)
        x = rng.standard_normal((ROWS * ROWS, 24)).astype(np.float32)
        mlp = WS.load_mlp(local) if os.path.exists(WS.WEIGHTS) else N.Mlp(seed=1, device=local)
        mlp.forward(x)
        t0 = time.perf_counter()
        for _ in range(5):
            mlp.forward(x)
        out["mlp_inference_spring_cloth_513"] = {"rows": ROWS * ROWS, "ms_per_call_with_copies":
                                                 1e3 * (time.perf_counter() - t0) / 5}
        mlp.close()
    if want("mesh_input"):
        out["mesh_input"] = mesh_input()
    if want("topology_change"):
        out["topology_change"] = topology_change(local)
    return out


def topology_change(local) -> dict:
    """Setup costs on a topology change of the 513x513 cloth: creating a solver (colouring,
    layout, tiles, with and without the launch autotuner), a pick (dynamic anchor) added
    between steps, and the energies' precomputations and incidence lists on the host against
    the GPU. Wall times on the host, median of three."""
    from spg_gb300 import native as N
    from spg_gb300 import scenes as S

    def med(fn, reps=3):
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return 1e3 * statistics.median(ts)

    obj = S.spring_cloth(ROWS).objects[0]
    out = {}
    kw = dict(dt=DT, iterations=ITERATIONS, gravity=GRAVITY, device=local)
    t0 = time.perf_counter()
    s = N.VbdSolver([obj], **kw)
    out["create_autotuned_ms"] = 1e3 * (time.perf_counter() - t0)
    k, g, b = s.launch()
    fixed = dict(kernel=k, lanes_per_vertex=g, block_size=b if k == 1 else 0, tile_vertices=b // g if k >= 2 else 0)
    s.close()

    def create_fixed():
        N.VbdSolver([obj], **kw, **fixed).close()

    out["create_fixed_launch_ms"] = med(create_fixed)
    s = N.VbdSolver([obj], **kw, **fixed)
    for _ in range(3):
        s.step()
    plain = statistics.median(s.step().device_ms for _ in range(3))
    v = obj.nv - 1
    x = s.state(0)[0][v]
    out["pick_add_ms"] = med(lambda: (s.set_picks([(0, v, x + 0.01, 1e4)]), s.set_picks([])))
    s.set_picks([(0, v, x + 0.01, 1e4)])
    s.step()
    picked = statistics.median(s.step().device_ms for _ in range(3))
    out["step_ms_without_pick"], out["step_ms_with_pick"] = plain, picked
    s.close()
    bend = next(e for e in obj.energies if e.type == N.BENDING)
    springs = next(e for e in obj.energies if e.type == N.SPRING)
    for name, e, mat in (("bending", bend, [0.0, 1e-4]), ("springs", springs, [0.0, 1e4])):
        m = np.asarray(mat, np.float64)
        host = med(lambda: N.precompute_params(e.type, e.stencils, obj.x0, m, device=None))
        dev = med(lambda: N.precompute_params(e.type, e.stencils, obj.x0, m, device=local))
        out[f"precompute_{name}"] = {"stencils": e.n, "host_ms": host, "gpu_ms": dev}
    host = med(lambda: N.incidences(obj))
    dev = med(lambda: N.incidences(obj, device=local))
    out["incidences"] = {"entries": int(sum(e.n * e.stencils.shape[1] for e in obj.energies)), "host_ms": host,
                         "gpu_ms": dev}
    return out


def mesh_input() -> dict:
    """Host mesh readers (spg::io::loadObj / loadMsh) on files written from the benchmark
    meshes: the 513x513 cloth as OBJ and an 81x21x21 six-tet bar as MSH 4.1 (ASCII and
    binary). Median wall time of three reads each."""
    import tempfile

    from spg_gb300 import scenes as S
    from tests import meshfiles as MF

    def faces(n):
        """The triangles of the grid builder (alternating diagonals), row by row."""
        r, c = (a.ravel() for a in np.meshgrid(np.arange(1, n), np.arange(1, n), indexing="ij"))
        even = ((r + c) % 2 == 0)[:, None]
        ll, ul, ur, lr = r * n + c - 1, (r - 1) * n + c - 1, (r - 1) * n + c, r * n + c
        t1 = np.where(even, np.stack([ll, ul, ur], 1), np.stack([ul, lr, ll], 1))
        t2 = np.where(even, np.stack([ll, ur, lr], 1), np.stack([ul, ur, lr], 1))
        return np.stack([t1, t2], 1).reshape(-1, 3)

    def timed(fn, path):
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            V, C = fn(path)
            ts.append(time.perf_counter() - t0)
        ms = 1e3 * statistics.median(ts)
        return {"ms": ms, "mb_per_s": os.path.getsize(path) / 1e6 / (ms * 1e-3), "vertices": len(V), "cells": len(C),
                "file_mb": os.path.getsize(path) / 1e6}

    out = {}
    with tempfile.TemporaryDirectory() as d:
        cloth = S.spring_cloth(ROWS).objects[0]
        p = os.path.join(d, "cloth.obj")
        MF.write_obj(p, cloth.x0, faces(ROWS))
        out["obj_cloth_513"] = timed(S.load_obj, p)
        bar = S.tet_beam(81, 21, 21).objects[0]
        T = next(e for e in bar.energies if e.stencils.shape[1] == 4).stencils
        for binary in (False, True):
            q = os.path.join(d, f"bar_{int(binary)}.msh")
            MF.write_msh41(q, bar.x0, T, binary=binary, node_blocks=4)
            out["msh41_bar_81x21x21_" + ("binary" if binary else "ascii")] = timed(S.load_msh, q)
    out["threads"] = 1
    return out


def run_reference(args, dist, rank, local, ws):
    if rank != 0:
        return 0
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    w = 2.0
    obj = O.build_spring_cloth(0.1 * w * w, w, w, ROWS, ROWS, 1e4, 1e-4, 1e5, 0.1, 12345)
    s = O.Vbd(obj, DT, 1, ITERATIONS, GRAVITY, O.FULL_AD)
    s.begin_substep()
    ncol = s.n_colors()
    for k in range(args.warmup):
        s.iterate_color(k % ncol)
    times, done = [], 0
    for k in range(args.steps):
        c = (args.warmup + k) % ncol
        t0 = time.perf_counter()
        s.iterate_color(c)
        times.append(time.perf_counter() - t0)
        done += s.color_size(c)
    total = sum(times)
    value = done / total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "parallelism": "host OpenMP"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step = one colour phase of one VBD iteration (colours cycled), "
                                       f"{done} vertex-solves in total, full-element FP64 AD per incidence"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, dist, rank, local, ws):
    import numpy as np

    from spg_gb300 import native as N
    from spg_gb300 import scenes as S

    scene = S.spring_cloth(ROWS)
    obj = scene.objects[0]
    solver = N.VbdSolver([obj], dt=DT, iterations=ITERATIONS, gravity=GRAVITY, device=local,
                         lanes_per_vertex=args.lanes, block_size=args.block, kernel=args.kernel,
                         tile_vertices=args.tile)
    kernel, lanes, block = solver.launch()
    nv = obj.nv

    import torch
    dev = torch.device(f"cuda:{local}")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2

    for _ in range(args.warmup):
        solver.step()
    sampler = ClockSampler(local)
    _barrier(dist, local)
    torch.cuda.synchronize(dev)
    sampler.start()
    t_wall0 = time.perf_counter()
    dev_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize(dev)
        st = solver.step()
        dev_ms.append(st.device_ms)
    torch.cuda.synchronize(dev)
    _barrier(dist, local)
    wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    dev_total_s = _max_over_ranks(dist, local, sum(dev_ms) * 1e-3)
    solves = _sum_over_ranks(dist, local, float(nv * ITERATIONS * args.steps))
    value = solves / dev_total_s
    # substep kernels + colour launches (one dataflow launch covers all sweeps of a step)
    launches_per_step = 2 + (1 if kernel == 3 else ITERATIONS * solver.n_colors(-1))

    # End-to-end through the C ABI with pinned FP64 host buffers (the ParticleGroup positions
    # and velocities a caller holds): upload state, step, download state.
    import torch
    x_host = torch.empty((nv, 3), dtype=torch.float64, pin_memory=True).numpy()
    v_host = torch.empty((nv, 3), dtype=torch.float64, pin_memory=True).numpy()
    solver.get_state_into(0, x_host, v_host)
    e2e_steps = max(1, min(args.steps, 10))
    _barrier(dist, local)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.set_state(0, x_host, v_host)
        solver.step()
        solver.get_state_into(0, x_host, v_host)
    _barrier(dist, local)
    e2e_s = _max_over_ranks(dist, local, time.perf_counter() - t0)
    e2e_value = _sum_over_ranks(dist, local, float(nv * ITERATIONS * e2e_steps)) / e2e_s
    bytes_state = nv * 6 * 8  # FP64 positions and velocities per vertex, each way

    # Roofline of the dominant kernel (the per-colour VBD kernel, 99 % of the device time in the
    # ncu launch list): the CUDA-event time of the timed steps on the solver's stream, divided
    # by the colour sweeps they ran. The two O(V) substep kernels stay in the denominator, so
    # the figure is a slight underestimate. The per-colour times of separately event-timed
    # launches (no overlap between launches) are reported beside it.
    sweep_s = dev_total_s / (args.steps * ITERATIONS)
    color_ms = solver.profile_sweeps(5)
    alg_bytes = algorithmic_bytes_per_iteration(obj)
    peak, peak_kind = _measured_peaks()
    achieved = alg_bytes / sweep_s / 1e9
    kernel_name = {1: "vbd_color_kernel", 2: "vbd_tile_kernel", 3: "vbd_flow_kernel"}[kernel]
    traffic = _traffic_per_iteration(kernel_name)

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_total_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "l2": "flushed between timed steps (256 MiB write)",
                   "kernel": {1: "lanes-per-vertex", 2: "shared-memory tiles, one launch per colour",
                              3: "shared-memory tiles, dataflow (one persistent launch per step)"}[kernel],
                   "lanes_per_vertex": lanes, "block_size": block,
                   "tile_vertices": block // lanes if kernel >= 2 else None,
                   "colors": int(solver.n_colors(-1)),
                   "parallelism": "replicas" if ws > 1 else "single GPU", "wall_s_timed_region": wall},
        "gpu_launches": launches_per_step * args.steps,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                "steps": e2e_steps, "host_buffers": "pinned FP64 positions and velocities"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind,
                     "kernel": kernel_name,
                     "algorithmic_bytes_per_sweep": alg_bytes,
                     "bytes_per_vertex_solve": alg_bytes / nv, "sweep_ms": 1e3 * sweep_s,
                     "launches_per_sweep": int(solver.n_colors(-1)),
                     "color_launch_ms_isolated": [round(float(c), 5) for c in color_ms]},
        "clocks": clocks,
    }
    ttr = None
    if not args.skip_extras:
        ttr = time_to_residual_legs(local)
        line["configs"] = other_configs(local)
    if ws == 1 and not args.skip_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if ttr is not None:
        line["time_to_residual"] = ttr  # last: the second half of the metric, kept by a log's tail
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--skip-cpu-baseline", action="store_true")
    ap.add_argument("--skip-extras", action="store_true", help="skip time-to-residual and the other configs")
    ap.add_argument("--lanes", type=int, default=0, help="lanes per vertex (0 = autotune)")
    ap.add_argument("--block", type=int, default=0, help="threads per block (0 = autotune)")
    ap.add_argument("--tile", type=int, default=0, help="vertices per tile of kernels 2 and 3 (0 = autotune)")
    ap.add_argument("--config", default=None,
                    help="run only this entry of the other configurations and print it (a profiling case)")
    ap.add_argument("--kernel", type=int, default=0,
                    help="1 = lanes per vertex, 2 = tiles, 3 = dataflow tiles (0 = autotune)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    dist, rank, local, ws = _dist()
    try:
        if args.config:
            import torch
            torch.cuda.set_device(local)
            print(json.dumps(other_configs(local, only=args.config)), flush=True)
            return 0
        if args.impl == "reference":
            return run_reference(args, dist, rank, local, ws)
        return run_gb300(args, dist, rank, local, ws)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
