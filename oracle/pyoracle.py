"""ctypes bindings of the oracle library (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module,
always as the checker or as the timed CPU restatement of the reference — never as the
product path.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

SPRING, ANCHOR, BENDING, STVK, SNH = 1, 2, 3, 4, 5
# Types 6-14: StVK tet, stable squared neo-Hookean, Baraff-Witkin membrane, Choi membrane,
# Baraff-Witkin bending, quadratic bending, continuum spring, squared continuum spring, load.
(STVK_TET, SSNH, BW_MEMBRANE, CHOI_MEMBRANE, BW_BENDING, QUAD_BENDING, SPRING_CONT, SPRING_SQ_CONT,
 STATIC_LOAD) = range(6, 15)
STENCIL_SIZE = {SPRING: 2, ANCHOR: 1, BENDING: 4, STVK: 3, SNH: 4, STVK_TET: 4, SSNH: 4, BW_MEMBRANE: 3,
                CHOI_MEMBRANE: 3, BW_BENDING: 4, QUAD_BENDING: 4, SPRING_CONT: 2, SPRING_SQ_CONT: 2, STATIC_LOAD: 1}
PARAM_COUNT = {SPRING: 3, ANCHOR: 5, BENDING: 3, STVK: 22, SNH: 14, STVK_TET: 13, SSNH: 13, BW_MEMBRANE: 10,
               CHOI_MEMBRANE: 12, BW_BENDING: 3, QUAD_BENDING: 6, SPRING_CONT: 3, SPRING_SQ_CONT: 3, STATIC_LOAD: 4}
FULL_AD, VERTEX_AD = 0, 1


class EnergyDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("n_stencils", C.c_int32),
                ("stencils", C.POINTER(C.c_int32)), ("params", C.POINTER(C.c_double))]


class ObjectDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("x", C.POINTER(C.c_double)), ("v", C.POINTER(C.c_double)),
                ("mass", C.POINTER(C.c_double)), ("n_energies", C.c_int32),
                ("energies", C.POINTER(EnergyDesc))]


@dataclass
class Energy:
    type: int
    stencils: np.ndarray  # int32 [n, S]
    params: np.ndarray    # float64 [n, P]

    @property
    def n(self) -> int:
        return int(self.stencils.shape[0])


@dataclass
class SceneObject:
    """One ParticleGroup: positions, velocities, masses and its energies in order."""
    x: np.ndarray      # float64 [V, 3]
    mass: np.ndarray   # float64 [V]
    energies: list = field(default_factory=list)
    v: np.ndarray | None = None
    x0: np.ndarray | None = None

    @property
    def nv(self) -> int:
        return int(self.mass.shape[0])

    def copy(self) -> "SceneObject":
        return SceneObject(self.x.copy(), self.mass.copy(),
                           [Energy(e.type, e.stencils.copy(), e.params.copy()) for e in self.energies],
                           None if self.v is None else self.v.copy(),
                           None if self.x0 is None else self.x0.copy())


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class _Desc:
    """Keeps numpy buffers alive for as long as the ctypes descriptor is used."""

    def __init__(self, obj: SceneObject):
        self.keep = []
        x = np.ascontiguousarray(obj.x, dtype=np.float64)
        m = np.ascontiguousarray(obj.mass, dtype=np.float64)
        v = None if obj.v is None else np.ascontiguousarray(obj.v, dtype=np.float64)
        self.keep += [x, m, v]
        es = (EnergyDesc * max(1, len(obj.energies)))()
        for i, e in enumerate(obj.energies):
            st = np.ascontiguousarray(e.stencils, dtype=np.int32)
            pa = np.ascontiguousarray(e.params, dtype=np.float64)
            self.keep += [st, pa]
            es[i] = EnergyDesc(e.type, e.n, _ptr(st, C.c_int32), _ptr(pa, C.c_double))
        self.keep.append(es)
        self.desc = ObjectDesc(obj.nv, _ptr(x, C.c_double), None if v is None else _ptr(v, C.c_double),
                               _ptr(m, C.c_double), len(obj.energies), es)


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from oracle import build as _b
            _b.build()
        L = C.CDLL(path)
        vp, i32, f64, dp = C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_build_cloth.restype = vp
        L.oracle_build_cloth.argtypes = [f64, C.c_float, C.c_float, i32, i32, f64, f64, f64, f64, i32, i32, ip]
        L.oracle_build_spring_cloth.restype = vp
        L.oracle_build_spring_cloth.argtypes = [f64, C.c_float, C.c_float, i32, i32, f64, f64, f64, f64, C.c_uint64]
        L.oracle_build_tet_beam.restype = vp
        L.oracle_build_tet_beam.argtypes = [f64, C.c_float, C.c_float, C.c_float, i32, i32, i32, f64, f64, f64, i32]
        L.oracle_build_patch_batch.restype = i32
        L.oracle_build_patch_batch.argtypes = [i32, i32, i32, f64, f64, f64, f64, f64, f64, C.c_uint64,
                                               C.POINTER(vp)]
        L.oracle_object_free.argtypes = [vp]
        L.oracle_object_nv.argtypes = [vp]
        L.oracle_object_n_energies.argtypes = [vp]
        L.oracle_object_arrays.argtypes = [vp] + [C.POINTER(dp)] * 4
        L.oracle_object_energy.argtypes = [vp, i32, ip, ip, C.POINTER(ip), C.POINTER(dp)]
        L.oracle_vbd_create.restype = vp
        L.oracle_vbd_create.argtypes = [C.POINTER(ObjectDesc), f64, i32, i32, dp, i32]
        for name in ["oracle_vbd_free", "oracle_vbd_step", "oracle_vbd_begin_substep", "oracle_vbd_end_substep"]:
            getattr(L, name).argtypes = [vp]
        L.oracle_vbd_set_mode.argtypes = [vp, i32]
        L.oracle_vbd_iterate.argtypes = [vp, i32]
        L.oracle_vbd_iterate_color.argtypes = [vp, i32]
        L.oracle_vbd_get_state.argtypes = [vp, dp, dp]
        L.oracle_vbd_set_state.argtypes = [vp, dp, dp]
        L.oracle_vbd_get_inertial.argtypes = [vp, dp]
        L.oracle_vbd_n_colors.argtypes = [vp]
        L.oracle_vbd_color_size.argtypes = [vp, i32]
        L.oracle_vbd_colors.argtypes = [vp, ip]
        L.oracle_vbd_adjacency_size.restype = C.c_longlong
        L.oracle_vbd_adjacency_size.argtypes = [vp]
        L.oracle_vbd_adjacency.argtypes = [vp, ip, ip]
        L.oracle_vbd_residual.restype = f64
        L.oracle_vbd_residual.argtypes = [vp, dp]
        L.oracle_xpbd_create.restype = vp
        L.oracle_xpbd_create.argtypes = [C.POINTER(ObjectDesc), f64, i32, dp]
        L.oracle_xpbd_free.argtypes = [vp]
        L.oracle_xpbd_step.argtypes = [vp]
        L.oracle_xpbd_get_state.argtypes = [vp, dp, dp]
        L.oracle_xpbd_n_groups.argtypes = [vp, i32]
        L.oracle_xpbd_stencil_colors.argtypes = [vp, i32, ip]
        L.oracle_element_block.argtypes = [i32, dp, dp, i32, i32, dp, dp]
        L.oracle_element_energy.restype = f64
        L.oracle_element_energy.argtypes = [i32, dp, dp]
        L.oracle_element_full.argtypes = [i32, dp, dp, dp, dp]
        L.oracle_element_constraints.argtypes = [i32, dp, dp, dp, dp]
        L.oracle_n_constraints.argtypes = [i32]
        L.oracle_color_vertices.argtypes = [C.POINTER(ObjectDesc), ip]
        L.oracle_set_threads.argtypes = [i32]
        _lib = L
    return _lib


def _err() -> str:
    return lib().oracle_last_error().decode()


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _object_from_handle(h) -> SceneObject:
    L = lib()
    nv = L.oracle_object_nv(h)
    px, px0, pv, pm = (C.POINTER(C.c_double)() for _ in range(4))
    L.oracle_object_arrays(h, C.byref(px), C.byref(px0), C.byref(pv), C.byref(pm))
    x = np.ctypeslib.as_array(px, shape=(nv, 3)).copy()
    x0 = np.ctypeslib.as_array(px0, shape=(nv, 3)).copy()
    v = np.ctypeslib.as_array(pv, shape=(nv, 3)).copy()
    m = np.ctypeslib.as_array(pm, shape=(nv,)).copy()
    energies = []
    for e in range(L.oracle_object_n_energies(h)):
        t, n = C.c_int(), C.c_int()
        ps, pp = C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
        L.oracle_object_energy(h, e, C.byref(t), C.byref(n), C.byref(ps), C.byref(pp))
        S, P = STENCIL_SIZE[t.value], PARAM_COUNT[t.value]
        st = np.ctypeslib.as_array(ps, shape=(n.value * S,)).reshape(n.value, S).astype(np.int32) if n.value else \
            np.zeros((0, S), np.int32)
        pa = np.ctypeslib.as_array(pp, shape=(n.value * P,)).reshape(n.value, P).copy() if n.value else \
            np.zeros((0, P), np.float64)
        energies.append(Energy(t.value, st, pa))
    L.oracle_object_free(h)
    return SceneObject(x, m, energies, v, x0)


def build_cloth(mass, width, height, rows, cols, young, poisson, bend_k, anchor_k, rest_initial=True,
                anchors=None) -> SceneObject:
    L = lib()
    if anchors is None:
        h = L.oracle_build_cloth(mass, width, height, rows, cols, young, poisson, bend_k, anchor_k,
                                 int(rest_initial), -1, None)
    else:
        a = np.ascontiguousarray(anchors, dtype=np.int32)
        h = L.oracle_build_cloth(mass, width, height, rows, cols, young, poisson, bend_k, anchor_k,
                                 int(rest_initial), len(a), _ptr(a, C.c_int))
    if not h:
        raise RuntimeError(_err())
    return _object_from_handle(h)


def build_spring_cloth(mass, width, height, rows, cols, spring_k, bend_k, anchor_k, jitter, seed) -> SceneObject:
    h = lib().oracle_build_spring_cloth(mass, width, height, rows, cols, spring_k, bend_k, anchor_k, jitter, seed)
    if not h:
        raise RuntimeError(_err())
    return _object_from_handle(h)


def build_tet_beam(mass, sx, sy, sz, nx, ny, nz, young, poisson, anchor_k, split=6) -> SceneObject:
    h = lib().oracle_build_tet_beam(mass, sx, sy, sz, nx, ny, nz, young, poisson, anchor_k, split)
    if not h:
        raise RuntimeError(_err())
    return _object_from_handle(h)


def build_patch_batch(n_patches, n_min, n_max, mu_lo, mu_hi, kb_lo, kb_hi, mass, anchor_k, seed) -> list:
    hs = (C.c_void_p * n_patches)()
    if lib().oracle_build_patch_batch(n_patches, n_min, n_max, mu_lo, mu_hi, kb_lo, kb_hi, mass, anchor_k, seed, hs):
        raise RuntimeError(_err())
    return [_object_from_handle(h) for h in hs]


class Vbd:
    """FP64 restatement of spg::solver::VBD on one object."""

    def __init__(self, obj: SceneObject, dt, substeps, iterations, gravity, mode=VERTEX_AD):
        self._d = _Desc(obj)
        g = np.ascontiguousarray(gravity, dtype=np.float64)
        self.h = lib().oracle_vbd_create(C.byref(self._d.desc), dt, substeps, iterations, _ptr(g, C.c_double), mode)
        if not self.h:
            raise RuntimeError(_err())
        self.nv = obj.nv
        self.dt, self.substeps = dt, substeps

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_vbd_free(self.h)
            self.h = None

    def set_mode(self, mode):
        lib().oracle_vbd_set_mode(self.h, mode)

    def step(self):
        lib().oracle_vbd_step(self.h)

    def begin_substep(self):
        lib().oracle_vbd_begin_substep(self.h)

    def iterate(self, n=1):
        lib().oracle_vbd_iterate(self.h, n)

    def iterate_color(self, c):
        lib().oracle_vbd_iterate_color(self.h, c)

    def end_substep(self):
        lib().oracle_vbd_end_substep(self.h)

    def state(self):
        x = np.zeros((self.nv, 3))
        v = np.zeros((self.nv, 3))
        lib().oracle_vbd_get_state(self.h, _ptr(x, C.c_double), _ptr(v, C.c_double))
        return x, v

    def set_state(self, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().oracle_vbd_set_state(self.h, _ptr(x, C.c_double), _ptr(v, C.c_double))

    def inertial(self):
        y = np.zeros((self.nv, 3))
        lib().oracle_vbd_get_inertial(self.h, _ptr(y, C.c_double))
        return y

    def colors(self):
        c = np.zeros(self.nv, np.int32)
        lib().oracle_vbd_colors(self.h, _ptr(c, C.c_int))
        return c

    def n_colors(self):
        return int(lib().oracle_vbd_n_colors(self.h))

    def color_size(self, c):
        return int(lib().oracle_vbd_color_size(self.h, c))

    def adjacency(self, n_energies):
        n = lib().oracle_vbd_adjacency_size(self.h)
        counts = np.zeros(self.nv * n_energies, np.int32)
        ent = np.zeros((max(1, n), 2), np.int32)
        lib().oracle_vbd_adjacency(self.h, _ptr(counts, C.c_int), _ptr(ent, C.c_int))
        return counts.reshape(self.nv, n_energies), ent[:n]

    def residual(self, per_component=False):
        if per_component:
            r = np.zeros((self.nv, 3))
            nrm = lib().oracle_vbd_residual(self.h, _ptr(r, C.c_double))
            return nrm, r
        return lib().oracle_vbd_residual(self.h, None)


class Xpbd:
    """FP64 restatement of spg::solver::XPBD on one object."""

    def __init__(self, obj: SceneObject, dt, substeps, gravity):
        self._d = _Desc(obj)
        g = np.ascontiguousarray(gravity, dtype=np.float64)
        self.h = lib().oracle_xpbd_create(C.byref(self._d.desc), dt, substeps, _ptr(g, C.c_double))
        if not self.h:
            raise RuntimeError(_err())
        self.nv = obj.nv
        self.n_energies = len(obj.energies)
        self.n_stencils = [e.n for e in obj.energies]

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_xpbd_free(self.h)
            self.h = None

    def step(self):
        lib().oracle_xpbd_step(self.h)

    def state(self):
        x = np.zeros((self.nv, 3))
        v = np.zeros((self.nv, 3))
        lib().oracle_xpbd_get_state(self.h, _ptr(x, C.c_double), _ptr(v, C.c_double))
        return x, v

    def stencil_colors(self, e):
        out = np.zeros(self.n_stencils[e], np.int32)
        lib().oracle_xpbd_stencil_colors(self.h, e, _ptr(out, C.c_int))
        return out


def element_block(etype, X, params, slot, mode=FULL_AD):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(params, dtype=np.float64)
    g = np.zeros(3)
    H = np.zeros(9)
    if lib().oracle_element_block(etype, _ptr(X, C.c_double), _ptr(p, C.c_double), slot, mode,
                                  _ptr(g, C.c_double), _ptr(H, C.c_double)):
        raise RuntimeError(_err())
    return g, H.reshape(3, 3)


def element_energy(etype, X, params) -> float:
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(params, dtype=np.float64)
    return float(lib().oracle_element_energy(etype, _ptr(X, C.c_double), _ptr(p, C.c_double)))


def element_full(etype, X, params):
    S = STENCIL_SIZE[etype]
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(params, dtype=np.float64)
    g = np.zeros(3 * S)
    H = np.zeros((3 * S, 3 * S))
    lib().oracle_element_full(etype, _ptr(X, C.c_double), _ptr(p, C.c_double), _ptr(g, C.c_double),
                              _ptr(H, C.c_double))
    return g, H


def element_constraints(etype, X, params):
    S = STENCIL_SIZE[etype]
    nc = lib().oracle_n_constraints(etype)
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(params, dtype=np.float64)
    c = np.zeros(nc)
    g = np.zeros(nc * 3 * S)
    lib().oracle_element_constraints(etype, _ptr(X, C.c_double), _ptr(p, C.c_double), _ptr(c, C.c_double),
                                     _ptr(g, C.c_double))
    return c, g.reshape(nc, 3 * S)


def color_vertices(obj: SceneObject) -> np.ndarray:
    d = _Desc(obj)
    out = np.zeros(obj.nv, np.int32)
    if lib().oracle_color_vertices(C.byref(d.desc), _ptr(out, C.c_int)):
        raise RuntimeError(_err())
    return out


# ---- the reference's own colouring, compiled from its sources ---------------------------
_ref = None


def ref_lib():
    """Loads oracle/_ref/libref_coloring.so, or returns None when it was not built."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libref_coloring.so")
        if not os.path.exists(path):
            return None
        R = C.CDLL(path)
        R.ref_color_vertices.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.c_int)]
        R.ref_color_stencils.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _ref = R
    return _ref


def ref_color_vertices(obj: SceneObject) -> np.ndarray:
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference colouring library not built")
    n = len(obj.energies)
    sizes = (C.c_int * max(1, n))(*[STENCIL_SIZE[e.type] for e in obj.energies])
    flats = [np.ascontiguousarray(e.stencils.reshape(-1), dtype=np.int32) for e in obj.energies]
    counts = (C.c_int * max(1, n))(*[len(f) for f in flats])
    ptrs = (C.POINTER(C.c_int) * max(1, n))(*[_ptr(f, C.c_int) for f in flats])
    out = np.zeros(obj.nv, np.int32)
    if R.ref_color_vertices(obj.nv, n, sizes, counts, ptrs, _ptr(out, C.c_int)):
        raise RuntimeError("reference colorVertices threw")
    return out


def ref_color_stencils(e: Energy) -> np.ndarray:
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference colouring library not built")
    flat = np.ascontiguousarray(e.stencils.reshape(-1), dtype=np.int32)
    out = np.zeros(e.n, np.int32)
    if R.ref_color_stencils(STENCIL_SIZE[e.type], len(flat), _ptr(flat, C.c_int), _ptr(out, C.c_int)):
        raise RuntimeError("reference colorStencils threw")
    return out
