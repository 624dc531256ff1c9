"""Benchmark scenes built by the library's own C++ scene builders (include/spgx_scenes.h)."""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from spg_gb300 import native as N

GRAVITY = (0.0, 0.0, -9.81)


@dataclass
class Energy:
    type: int
    stencils: np.ndarray
    params: np.ndarray

    @property
    def n(self) -> int:
        return int(self.stencils.shape[0])


@dataclass
class SceneObject:
    x: np.ndarray
    mass: np.ndarray
    energies: list = field(default_factory=list)
    v: np.ndarray | None = None
    x0: np.ndarray | None = None

    @property
    def nv(self) -> int:
        return int(self.mass.shape[0])


_bound = False


def _lib():
    global _bound
    L = N.lib()
    if not _bound:
        vp, i32, f64, f32 = C.c_void_p, C.c_int32, C.c_double, C.c_float
        L.spgx_scene_cloth.argtypes = [f64, f32, f32, i32, i32, f64, f64, f64, f64, i32, C.POINTER(i32), i32,
                                       C.POINTER(vp)]
        L.spgx_scene_spring_cloth.argtypes = [f64, f32, f32, i32, i32, f64, f64, f64, f64, C.c_uint64, C.POINTER(vp)]
        L.spgx_scene_tet_beam.argtypes = [f64, f32, f32, f32, i32, i32, i32, f64, f64, f64, i32, C.POINTER(vp)]
        L.spgx_scene_patch_batch.argtypes = [i32, i32, i32, f64, f64, f64, f64, f64, f64, C.c_uint64, C.POINTER(vp)]
        L.spgx_scene_get_desc.argtypes = [vp, C.POINTER(C.POINTER(N.SceneDesc))]
        L.spgx_scene_rest_positions.argtypes = [vp, i32, C.POINTER(f64)]
        L.spgx_scene_destroy.argtypes = [vp]
        L.spgx_scene_run_gpu_vbd.argtypes = [vp, C.POINTER(N.VbdParams), i32, C.POINTER(f64)]
        L.spgx_scene_run_gpu_xpbd.argtypes = [vp, C.POINTER(N.XpbdParams), i32, C.POINTER(f64)]
        L.spgx_scene_run_gpu_implicit.argtypes = [vp, C.POINTER(N.ImplicitParams), i32, C.POINTER(f64)]
        pi = C.POINTER(i32)
        L.spgx_scene_triangle_mesh.argtypes = [C.POINTER(f64), i32, pi, i32, f64, f64, f64, f64, i32, pi,
                                               C.POINTER(vp)]
        L.spgx_scene_tet_mesh.argtypes = [C.POINTER(f64), i32, pi, i32, f64, f64, f64, f64, i32, pi, C.POINTER(vp)]
        L.spgx_load_obj.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.spgx_load_msh.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.spgx_mesh_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), pi]
        L.spgx_mesh_copy.argtypes = [vp, C.POINTER(f64), pi]
        L.spgx_mesh_destroy.argtypes = [vp]
        _bound = True
    return L


class Scene:
    """Owns an spgx_scene handle; `objects` copies its packed descriptor into numpy arrays."""

    def __init__(self, handle):
        self.h = handle
        L = _lib()
        pd = C.POINTER(N.SceneDesc)()
        N.check(L.spgx_scene_get_desc(self.h, C.byref(pd)))
        d = pd.contents
        self.objects = []
        for k in range(d.n_objects):
            ob = d.objects[k]
            nv = ob.n_vertices
            x = np.ctypeslib.as_array(ob.x, shape=(nv * 3,)).reshape(nv, 3).copy()
            v = np.ctypeslib.as_array(ob.v, shape=(nv * 3,)).reshape(nv, 3).copy()
            m = np.ctypeslib.as_array(ob.mass, shape=(nv,)).copy()
            x0 = np.zeros((nv, 3))
            N.check(L.spgx_scene_rest_positions(self.h, k, x0.ctypes.data_as(C.POINTER(C.c_double))))
            energies = []
            for i in range(ob.n_energies):
                e = ob.energies[i]
                S, P = N.STENCIL_SIZE[e.type], N.PARAM_COUNT[e.type]
                n = e.n_stencils
                st = np.ctypeslib.as_array(e.stencils, shape=(n * S,)).reshape(n, S).copy() if n else \
                    np.zeros((0, S), np.int32)
                pa = np.ctypeslib.as_array(e.params, shape=(n * P,)).reshape(n, P).copy() if n else \
                    np.zeros((0, P))
                energies.append(Energy(e.type, st, pa))
            self.objects.append(SceneObject(x, m, energies, v, x0))

    def close(self):
        if getattr(self, "h", None):
            _lib().spgx_scene_destroy(self.h)
            self.h = None

    __del__ = close

    def run_gpu_vbd(self, steps, **params):
        """Runs spg::solver::GpuVBD (the C++ drop-in class) and returns object 0's positions."""
        p = N.vbd_params(**params)
        out = np.zeros((self.objects[0].nv, 3))
        N.check(_lib().spgx_scene_run_gpu_vbd(self.h, C.byref(p), steps, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def run_gpu_implicit(self, steps, dt, substeps, gravity, method):
        """Runs spg::solver::GpuImplicit (the given global solver) and returns object 0's positions."""
        p = N.ImplicitParams()
        N.lib().spgx_implicit_params_default(C.byref(p))
        p.dt, p.substeps, p.method = dt, substeps, method
        p.gravity = (C.c_double * 3)(*gravity)
        out = np.zeros((self.objects[0].nv, 3))
        N.check(_lib().spgx_scene_run_gpu_implicit(self.h, C.byref(p), steps,
                                                   out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def run_gpu_xpbd(self, steps, dt, substeps, gravity):
        p = N.XpbdParams()
        N.lib().spgx_xpbd_params_default(C.byref(p))
        p.dt, p.substeps = dt, substeps
        p.gravity = (C.c_double * 3)(*gravity)
        out = np.zeros((self.objects[0].nv, 3))
        N.check(_lib().spgx_scene_run_gpu_xpbd(self.h, C.byref(p), steps, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out


def _make(fn, *args) -> Scene:
    h = C.c_void_p()
    N.check(fn(*args, C.byref(h)))
    return Scene(h)


def stvk_from_lame(mu: float, lam: float):
    """(young, poisson) whose plane-stress StVK matrix has c11 = 2 mu + lambda, c12 = lambda,
    c33 = mu."""
    nu = lam / (2 * mu + lam)
    return (2 * mu + lam) * (1 - nu * nu), nu


def cloth(rows=33, cols=None, mass=0.1, width=1.0, height=1.0, mu=1e4, lam=1e4, bending=1e-3, anchor_k=1e5,
          anchors=None, rest_initial=True) -> Scene:
    cols = rows if cols is None else cols
    young, nu = stvk_from_lame(mu, lam)
    if anchors is None:
        return _make(_lib().spgx_scene_cloth, mass, width, height, rows, cols, young, nu, bending, anchor_k, -1, None,
                     int(rest_initial))
    a = (C.c_int32 * len(anchors))(*anchors)
    return _make(_lib().spgx_scene_cloth, mass, width, height, rows, cols, young, nu, bending, anchor_k, len(anchors),
                 a, int(rest_initial))


def spring_cloth(n=513, spring_k=1e4, bending=1e-4, anchor_k=1e5, jitter=0.1, seed=12345, density=0.1) -> Scene:
    """Large-cloth spacing: 2 m at 513 vertices per side (edge 3.906 mm)."""
    w = 2.0 * (n - 1) / 512
    return _make(_lib().spgx_scene_spring_cloth, density * w * w, w, w, n, n, spring_k, bending, anchor_k, jitter, seed)


def tet_beam(nx=41, ny=11, nz=11, cell=0.025, density=1000.0, young=1e6, poisson=0.45, anchor_k=1e4, split=6) -> Scene:
    sx, sy, sz = cell * (nx - 1), cell * (ny - 1), cell * (nz - 1)
    return _make(_lib().spgx_scene_tet_beam, density * sx * sy * sz, sx, sy, sz, nx, ny, nz, young, poisson,
                 anchor_k, split)


def patch_batch(n_patches=512, n_min=16, n_max=128, seed=2024, mu_lo=1e3, mu_hi=1e5, kb_lo=1e-5, kb_hi=1e-2,
                mass=0.1, anchor_k=1e5) -> Scene:
    return _make(_lib().spgx_scene_patch_batch, n_patches, n_min, n_max, mu_lo, mu_hi, kb_lo, kb_hi, mass, anchor_k,
                 seed)


def _load(fn, path):
    h = C.c_void_p()
    N.check(fn(os.fsencode(path), C.byref(h)))
    try:
        nv, nc, k = C.c_int64(), C.c_int64(), C.c_int32()
        N.check(_lib().spgx_mesh_info(h, C.byref(nv), C.byref(nc), C.byref(k)))
        V = np.zeros((nv.value, 3))
        cells = np.zeros((nc.value, k.value), np.int32)
        N.check(_lib().spgx_mesh_copy(h, V.ctypes.data_as(C.POINTER(C.c_double)),
                                      cells.ctypes.data_as(C.POINTER(C.c_int32))))
    finally:
        _lib().spgx_mesh_destroy(h)
    return V, cells


def load_obj(path):
    """spg::io::loadObj: (vertices (n, 3) float64 holding float values, triangles (m, 3))."""
    return _load(_lib().spgx_load_obj, path)


def load_msh(path):
    """spg::io::loadMsh: (nodes (n, 3) float64, tetrahedra (m, 4))."""
    return _load(_lib().spgx_load_msh, path)


def _mesh_args(V, cells, k, anchors):
    V = np.ascontiguousarray(V, np.float64).reshape(-1, 3)
    cells = np.ascontiguousarray(cells, np.int32).reshape(-1, k)
    a = np.ascontiguousarray([] if anchors is None else anchors, np.int32)
    pi = C.POINTER(C.c_int32)
    return ((V, cells, a), V.ctypes.data_as(C.POINTER(C.c_double)), len(V), cells.ctypes.data_as(pi), len(cells),
            len(a), a.ctypes.data_as(pi))


def triangle_mesh(V, F, mass=0.1, spring_k=1e4, bending=1e-4, anchor_k=1e5, anchors=None) -> Scene:
    """A shell on a triangle mesh: springs on every edge, bending on interior edges, anchors."""
    keep, v, nv, f, nf, na, a = _mesh_args(V, F, 3, anchors)
    return _make(_lib().spgx_scene_triangle_mesh, v, nv, f, nf, mass, spring_k, bending, anchor_k, na, a)


def tet_mesh(V, T, mass=1.0, young=1e6, poisson=0.45, anchor_k=1e4, anchors=None) -> Scene:
    """A solid on a tetrahedral mesh: Stable Neo-Hookean tets and anchors."""
    keep, v, nv, t, nt, na, a = _mesh_args(V, T, 4, anchors)
    return _make(_lib().spgx_scene_tet_mesh, v, nv, t, nt, mass, young, poisson, anchor_k, na, a)

