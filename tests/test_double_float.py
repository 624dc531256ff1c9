"""The double-float arithmetic of the CG's matrix-vector products (implicit.cu: split_df,
df_fma, df_add), restated in numpy float32 and checked against FP64.
- split: a = hi + lo with hi = fl32(a), lo = fl32(a - hi), 48 significant bits;
- product: ph = fl32(ah xh), its rounding error from an FMA, plus the cross terms ah xl + al xh;
- accumulation: Knuth's two-sum of the heads, tails gathered separately.
fmaf(a, b, c) is emulated as fl32(a b + c) in FP64: the product of two float32 values is exact
in FP64, so only the final rounding differs, by at most one float32 ulp of a small term."""
import numpy as np

f32 = np.float32


def split(a):
    hi = f32(a)
    return hi, f32(a - np.float64(hi))


def fmaf(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def df_fma(sh, sl, a, x):
    ph = f32(a[0] * x[0])
    pl = fmaf(a[0], x[1], fmaf(a[1], x[0], fmaf(a[0], x[0], -ph)))
    s = f32(sh + ph)
    bb = f32(s - sh)
    e = f32(f32(sh - f32(s - bb)) + f32(ph - bb))
    return s, f32(sl + f32(e + pl))


def test_split_keeps_48_bits():
    rng = np.random.default_rng(0)
    a = rng.normal(size=10000) * np.exp(rng.uniform(-30, 30, 10000))
    for v in a:
        hi, lo = split(v)
        assert abs((np.float64(hi) + np.float64(lo)) - v) <= 2.0 ** -47 * abs(v)


def test_row_products_reach_double_float_accuracy():
    """Rows of 117 products (13 blocks of 9 values), as on the 513^2 cloth, with mixed signs:
    the double-float sum stays within 2^-43 of the FP64 sum, relative to the sum of
    magnitudes (2^-44.6 measured); plain FP32 is about 2^-24 away."""
    rng = np.random.default_rng(1)
    worst_df, worst_fp32 = 0.0, 0.0
    for _ in range(300):
        A = rng.normal(size=117) * 10 ** rng.uniform(-2, 4)
        x = rng.normal(size=117) * 10 ** rng.uniform(-6, 0)
        sh, sl = f32(0), f32(0)
        for a, v in zip(A, x):
            sh, sl = df_fma(sh, sl, split(a), split(v))
        exact = float(np.dot(A, x))
        scale = float(np.dot(np.abs(A), np.abs(x)))
        worst_df = max(worst_df, abs(np.float64(sh) + np.float64(sl) - exact) / scale)
        fp32 = float(np.dot(A.astype(f32), x.astype(f32)))
        worst_fp32 = max(worst_fp32, abs(fp32 - exact) / scale)
    assert worst_df < 2.0 ** -43
    assert worst_fp32 > 2.0 ** -30
