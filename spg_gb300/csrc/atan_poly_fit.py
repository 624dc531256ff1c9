"""Fits the polynomial behind the FP32 device arctan2 in elements.cuh.

atan(t) = t P(t^2) on [0, 1], P of degree 8, minimax in relative error by the Remez exchange
algorithm (E. Remez, 1934) on a dense grid. Prints the coefficients as float32 literals and
the largest error of the float32 Horner evaluation, in ulp of atan(t), over 2e6 points.
Run: python spg_gb300/csrc/atan_poly_fit.py
"""
import numpy as np

DEGREE = 8


def target(s):
    r = np.sqrt(np.maximum(s, 1e-300))
    return np.where(s > 0, np.arctan(r) / r, 1.0)


def remez(d, iterations=30):
    n = d + 2
    k = np.arange(n)
    ref = 0.5 - 0.5 * np.cos(np.pi * k / (n - 1))
    grid = np.linspace(0.0, 1.0, 200001)
    for _ in range(iterations):
        A = np.zeros((n, n))
        for j in range(d + 1):
            A[:, j] = ref ** j
        A[:, d + 1] = (-1.0) ** k * target(ref)
        c = np.linalg.solve(A, target(ref))[: d + 1]
        err = (np.polyval(c[::-1], grid) - target(grid)) / target(grid)
        segments = np.split(np.arange(grid.size), np.where(np.diff(np.sign(err)) != 0)[0] + 1)
        extrema = [seg[np.argmax(np.abs(err[seg]))] for seg in segments]
        if len(extrema) >= n:
            windows = [extrema[i:i + n] for i in range(len(extrema) - n + 1)]
            ref = grid[max(windows, key=lambda w: np.min(np.abs(err[w])))]
    return c


def float32_ulp_error(c32):
    t = np.linspace(0.0, 1.0, 2000001).astype(np.float32)
    s = t * t
    p = np.full_like(s, c32[-1])
    for cj in c32[-2::-1]:
        p = (p * s + cj).astype(np.float32)
    r = (t * p).astype(np.float64)
    exact = np.arctan(t.astype(np.float64))
    return float(np.max(np.abs(r - exact) / np.spacing(np.maximum(exact, 1e-30).astype(np.float32))))


if __name__ == "__main__":
    c32 = remez(DEGREE).astype(np.float32)
    print(", ".join(f"{float(v)!r}f" for v in c32))
    print(f"max error of the float32 evaluation: {float32_ulp_error(c32):.2f} ulp")
