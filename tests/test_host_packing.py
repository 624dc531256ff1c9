"""The C++ host layer (spg_gb300/host: the reference's energy classes without Eigen) sets up
the nine further energies and packs them into the C ABI exactly as the numpy restatement of
the reference's addStencil + preparePrecomputations does (CPU only)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

LIB = os.path.join(os.path.dirname(__file__), "native", "libhost_packing.so")


@pytest.fixture(scope="module")
def host():
    if not os.path.exists(LIB):
        import __graft_entry__ as ge
        ge._build_test_helpers()
    return C.CDLL(LIB)


def _pack(host, etype, x0, stencils, args):
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    st = np.ascontiguousarray(stencils, dtype=np.int32)
    a = np.ascontiguousarray(args, dtype=np.float64)
    n = st.shape[0]
    out = np.zeros(n * O.PARAM_COUNT[etype])
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    rc = host.host_pack(etype, x0.shape[0], x0.ctypes.data_as(dp), n, st.ctypes.data_as(ip), a.ctypes.data_as(dp),
                        out.ctypes.data_as(dp))
    assert rc == 0
    return out.reshape(n, -1)


def test_tet_energies(host):
    b = scenes.beam_cfg2(5, 3, 3)
    tets = next(e for e in b.energies if e.type == O.SNH).stencils
    ref = scenes.tet_params(b.x0, tets, 1e6, 0.45)
    for etype in (O.STVK_TET, O.SSNH):
        got = _pack(host, etype, b.x0, tets, [1e6, 0.45])
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-13 * np.abs(ref).max())


def test_membranes_and_bendings(host):
    c = scenes.cloth_cfg1(7)
    tris = next(e for e in c.energies if e.type == O.STVK).stencils
    bend = next(e for e in c.energies if e.type == O.BENDING).stencils
    got = _pack(host, O.BW_MEMBRANE, c.x0, tris, [1e3, 2e3, 5e2])
    assert np.allclose(got, scenes.membrane_params(c.x0, tris, [1e3, 2e3, 5e2]), rtol=1e-12)
    got = _pack(host, O.CHOI_MEMBRANE, c.x0, tris, [1e3, 2e3, 5e2])
    assert np.allclose(got, scenes.membrane_params(c.x0, tris, [1e3, 2e3, 5e2, 5e2]), rtol=1e-12)
    got = _pack(host, O.BW_BENDING, c.x0, bend, [1e-3])
    assert np.allclose(got, scenes.bw_bending_params(c.x0, bend, 1e-3), rtol=1e-12, atol=1e-15)
    got = _pack(host, O.QUAD_BENDING, c.x0, bend, [1e-3])
    assert np.allclose(got, scenes.quad_bending_params(c.x0, bend, 1e-3), rtol=1e-12, atol=1e-15)


def test_springs_and_load(host):
    s = scenes.spring_cloth_cfg3(5)
    pairs = next(e for e in s.energies if e.type == O.SPRING).stencils
    ref = scenes.continuum_spring_params(s.x0, pairs, 5e3)
    for etype in (O.SPRING_CONT, O.SPRING_SQ_CONT):
        assert np.allclose(_pack(host, etype, s.x0, pairs, [5e3]), ref, rtol=1e-12)
    got = _pack(host, O.STATIC_LOAD, s.x0, np.array([[0], [3]]), [2.0, 0.0, 3.0, 4.0])
    assert np.allclose(got, [[2.0, 0.0, 0.6, 0.8]] * 2)
