"""The solver's closed-form per-vertex blocks (spg_gb300/csrc/elements.cuh), instantiated on
the CPU in FP64 and FP32 by tests/native/elements_host.cpp, against the oracle's
full-element AD (the reference's derivative path)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

LIB = os.path.join(os.path.dirname(__file__), "native", "libelements_host.so")
dp = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def host():
    if not os.path.exists(LIB):
        import __graft_entry__ as ge
        ge._build_test_helpers()
    return C.CDLL(LIB)


def _block(fn, etype, X, p, slot):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(p, dtype=np.float64)
    g, H = np.zeros(3), np.zeros(9)
    fn(etype, X.ctypes.data_as(dp), p.ctypes.data_as(dp), slot, g.ctypes.data_as(dp), H.ctypes.data_as(dp))
    return g, H.reshape(3, 3)


def _cases():
    rng = np.random.default_rng(11)
    for obj in (scenes.cloth_cfg1(9), scenes.beam_cfg2(5, 3, 3), scenes.spring_cloth_cfg3(9)):
        scale = 0.02 * float(np.ptp(obj.x0, axis=0).max())
        for e in obj.energies:
            for i in rng.integers(0, e.n, size=min(25, e.n)):
                X = obj.x[e.stencils[i]] + rng.normal(scale=scale, size=(e.stencils.shape[1], 3))
                for slot in range(e.stencils.shape[1]):
                    yield e.type, X, e.params[i], slot


def test_fp64_closed_form_equals_full_element_ad(host):
    for etype, X, p, slot in _cases():
        g, H = _block(host.host_block_f64, etype, X, p, slot)
        gr, Hr = O.element_block(etype, X, p, slot, O.FULL_AD)
        assert np.abs(g - gr).max() <= 1e-9 * max(np.abs(gr).max(), 1e-300), (etype, slot)
        assert np.abs(H - Hr).max() <= 1e-9 * max(np.abs(Hr).max(), 1e-300), (etype, slot)


def test_fp32_closed_form_relative_error(host):
    """Same inputs rounded to FP32 for both: median relative error per block <= 1e-5."""
    eg, eh = [], []
    for etype, X, p, slot in _cases():
        X = X.astype(np.float32).astype(np.float64)
        p = p.astype(np.float32).astype(np.float64)
        g, H = _block(host.host_block_f32, etype, X, p, slot)
        gr, Hr = O.element_block(etype, X, p, slot, O.FULL_AD)
        eg.append(np.linalg.norm(g - gr) / max(np.linalg.norm(gr), 1e-300))
        eh.append(np.linalg.norm(H - Hr) / max(np.linalg.norm(Hr), 1e-300))
    assert np.median(eg) <= 1e-5 and np.median(eh) <= 1e-5
    assert np.quantile(eh, 0.99) <= 1e-5


def test_constraint_gradients_equal_oracle(host):
    nc = {O.ANCHOR: 1, O.BENDING: 1, O.STVK: 3, O.SNH: 2}
    for etype, X, p, slot in _cases():
        if etype == O.SPRING or slot:
            continue
        S = X.shape[0]
        c, G = np.zeros(nc[etype]), np.zeros(nc[etype] * 3 * S)
        Xf = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
        pf = np.ascontiguousarray(p, dtype=np.float64)
        host.host_constraints_f64(etype, Xf.ctypes.data_as(dp), pf.ctypes.data_as(dp), c.ctypes.data_as(dp),
                                  G.ctypes.data_as(dp))
        cr, Gr = O.element_constraints(etype, X, p)
        assert np.allclose(c, cr, rtol=1e-10, atol=1e-12)
        assert np.allclose(G.reshape(Gr.shape), Gr, rtol=1e-9, atol=1e-9 * max(1, np.abs(Gr).max()))
