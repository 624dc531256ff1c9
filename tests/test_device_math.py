"""Error bounds of the solver's FP32 device math (elements.cuh): the hardware approximate
reciprocal and the polynomial arctan2 used by the bending hinge angle, against FP64 on the
same FP32 inputs, with CUDA's own 1/x and atan2f run beside them for scale."""
import ctypes as C
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(y, x):
    path = os.path.join(HERE, "native", "libdevice_math.so")
    if not os.path.exists(path):
        pytest.fail("tests/native/libdevice_math.so is missing: run __graft_entry__.build()")
    lib = C.CDLL(path)
    fp = C.POINTER(C.c_float)
    lib.spgx_test_device_math.argtypes = [C.c_int, fp, fp, fp]
    y = np.ascontiguousarray(y, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((4, y.size), np.float32)
    assert lib.spgx_test_device_math(y.size, y.ctypes.data_as(fp), x.ctypes.data_as(fp), out.ctypes.data_as(fp)) == 0
    return out


def _inputs(n=2_000_000, seed=7):
    """Every octant, radii over 1e-17..1e17, and angles within 1e-3 of the octant borders
    (where the reduction switches branch) and of +-pi."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(-np.pi, np.pi, n)
    borders = np.arange(-4, 5) * (np.pi / 4)
    near = rng.choice(borders, n // 2) + rng.uniform(-1e-3, 1e-3, n // 2)
    ang = np.concatenate([ang, near])
    rad = np.exp(rng.uniform(-39, 39, ang.size))
    return (rad * np.sin(ang)).astype(np.float32), (rad * np.cos(ang)).astype(np.float32)


def _ulp(got, exact):
    return np.abs(got.astype(np.float64) - exact) / np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)


@pytest.mark.gpu
def test_arctan2_within_five_ulp():
    y, x = _inputs()
    ours, cuda, _, _ = _run(y, x)
    exact = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    e_ours, e_cuda = _ulp(ours, exact), _ulp(cuda, exact)
    print(f"arctan2: ours max {e_ours.max():.2f} ulp, atan2f max {e_cuda.max():.2f} ulp")
    assert e_ours.max() <= 5.0


@pytest.mark.gpu
def test_arctan2_signed_zeros_and_axes():
    y = np.array([0.0, -0.0, 0.0, -0.0, 1.0, -1.0, 0.0, 0.0, 1.0, -1.0, 3.0, -3.0], np.float32)
    x = np.array([0.0, 0.0, -0.0, -0.0, 0.0, 0.0, 2.0, -2.0, 1.0, -1.0, -3.0, 3.0], np.float32)
    ours, cuda, _, _ = _run(y, x)
    exact = np.arctan2(y.astype(np.float64), x.astype(np.float64)).astype(np.float32)
    assert np.all(np.signbit(ours) == np.signbit(exact))
    assert np.all(_ulp(ours, exact.astype(np.float64)) <= 1.0)


@pytest.mark.gpu
def test_reciprocal_within_one_ulp():
    rng = np.random.default_rng(3)
    x = (np.exp(rng.uniform(-80, 80, 1_000_000)) * rng.choice([-1.0, 1.0], 1_000_000)).astype(np.float32)
    _, _, ours, cuda = _run(np.zeros_like(x), x)
    exact = 1.0 / x.astype(np.float64)
    ok = np.abs(exact) < np.finfo(np.float32).max
    e = _ulp(ours[ok], exact[ok])
    print(f"reciprocal: max {e.max():.2f} ulp")
    assert e.max() <= 1.0
    assert np.isinf(_run(np.zeros(1), np.zeros(1))[2][0])


def test_arctan2_coefficients_are_the_fit_scripts_output():
    """The nine float32 literals of the device arctan2's polynomial (elements.cuh) are what
    atan_poly_fit.py beside it produces (Remez exchange, degree 8), bit for bit, and that
    polynomial's float32 Horner evaluation stays within 2 ulp of atan on [0, 1]."""
    import importlib.util
    import re
    csrc = os.path.join(os.path.dirname(HERE), "spg_gb300", "csrc")
    spec = importlib.util.spec_from_file_location("atan_poly_fit", os.path.join(csrc, "atan_poly_fit.py"))
    fit = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fit)
    c32 = fit.remez(fit.DEGREE).astype(np.float32)
    src = open(os.path.join(csrc, "elements.cuh")).read()
    body = src[src.index("SPGX_HD float arctan2(float y, float x)"):]
    body = body[:body.index("float r = t * p;")]
    lits = [float(v) for v in re.findall(r"p = (-?[0-9.e-]+)f;", body)]
    lits += [float(v) for v in re.findall(r"p = fmaf\(p, s, (-?[0-9.e-]+)f\);", body)]
    # highest degree first in the Horner chain; the script lists degree 0 first
    assert np.array_equal(np.array(lits[::-1], np.float32), c32)
    assert fit.float32_ulp_error(c32) <= 2.0
