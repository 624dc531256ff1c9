"""ctypes bindings of the C ABI in include/spgx.h (libspgx.so, built in-tree).

The solver itself is the CUDA library; this module only marshals descriptors and arrays.
Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libspgx.so")

SPRING, ANCHOR, BENDING, STVK, SNH = 1, 2, 3, 4, 5
# Types 6-14: StVK tet, stable squared neo-Hookean, Baraff-Witkin membrane, Choi membrane,
# Baraff-Witkin bending, quadratic bending, continuum spring, squared continuum spring, load.
(STVK_TET, SSNH, BW_MEMBRANE, CHOI_MEMBRANE, BW_BENDING, QUAD_BENDING, SPRING_CONT, SPRING_SQ_CONT,
 STATIC_LOAD) = range(6, 15)
STENCIL_SIZE = {SPRING: 2, ANCHOR: 1, BENDING: 4, STVK: 3, SNH: 4, STVK_TET: 4, SSNH: 4, BW_MEMBRANE: 3,
                CHOI_MEMBRANE: 3, BW_BENDING: 4, QUAD_BENDING: 4, SPRING_CONT: 2, SPRING_SQ_CONT: 2, STATIC_LOAD: 1}
PARAM_COUNT = {SPRING: 3, ANCHOR: 5, BENDING: 3, STVK: 22, SNH: 14, STVK_TET: 13, SSNH: 13, BW_MEMBRANE: 10,
               CHOI_MEMBRANE: 12, BW_BENDING: 3, QUAD_BENDING: 6, SPRING_CONT: 3, SPRING_SQ_CONT: 3, STATIC_LOAD: 4}

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "UNSUPPORTED_ENERGY", 3: "CUDA", 4: "NONFINITE", 5: "TIMEOUT",
          6: "NO_DEVICE"}


class SpgxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"spgx error {STATUS.get(status, status)}: {message}")
        self.status = status


class EnergyDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("n_stencils", C.c_int32),
                ("stencils", C.POINTER(C.c_int32)), ("params", C.POINTER(C.c_double))]


class ObjectDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("x", C.POINTER(C.c_double)), ("v", C.POINTER(C.c_double)),
                ("mass", C.POINTER(C.c_double)), ("n_energies", C.c_int32),
                ("energies", C.POINTER(EnergyDesc))]


class SceneDesc(C.Structure):
    _fields_ = [("n_objects", C.c_int32), ("objects", C.POINTER(ObjectDesc))]


class VbdParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("substeps", C.c_int32), ("iterations", C.c_int32),
                ("gravity", C.c_double * 3), ("tolerance", C.c_double), ("max_iterations", C.c_int32),
                ("check_interval", C.c_int32), ("fallback_condition", C.c_double),
                ("lanes_per_vertex", C.c_int32), ("block_size", C.c_int32), ("use_graph", C.c_int32),
                ("device", C.c_int32), ("kernel", C.c_int32), ("tile_vertices", C.c_int32)]


class XpbdParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("substeps", C.c_int32), ("gravity", C.c_double * 3),
                ("block_size", C.c_int32), ("use_graph", C.c_int32), ("device", C.c_int32),
                ("kernel", C.c_int32)]


class ImplicitParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("substeps", C.c_int32), ("gravity", C.c_double * 3),
                ("cg_threshold", C.c_double), ("cg_max_iterations", C.c_int32), ("device", C.c_int32),
                ("method", C.c_int32), ("cg_precision", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("fallback_solves", C.c_int32), ("skipped_solves", C.c_int32),
                ("converged", C.c_int32), ("residual_initial", C.c_double), ("residual_final", C.c_double),
                ("device_ms", C.c_double), ("warm_accepted", C.c_int32), ("extrapolated_accepted", C.c_int32),
                ("residual_warm", C.c_double), ("residual_extrapolated", C.c_double)]


_lib = None


def lib():
    """Loads libspgx.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        vp, i32, f64 = C.c_void_p, C.c_int32, C.c_double
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.spgx_last_error_string.restype = C.c_char_p
        L.spgx_api_version.restype = i32
        L.spgx_stencil_size.argtypes = [i32]
        L.spgx_param_count.argtypes = [i32]
        L.spgx_num_constraints.argtypes = [i32]
        L.spgx_vbd_params_default.argtypes = [C.POINTER(VbdParams)]
        L.spgx_xpbd_params_default.argtypes = [C.POINTER(XpbdParams)]
        L.spgx_vbd_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(VbdParams), C.POINTER(vp)]
        L.spgx_vbd_destroy.argtypes = [vp]
        L.spgx_vbd_set_params.argtypes = [vp, C.POINTER(VbdParams)]
        L.spgx_vbd_step.argtypes = [vp, C.POINTER(StepStats)]
        L.spgx_vbd_get_state.argtypes = [vp, i32, dp, dp]
        L.spgx_vbd_set_state.argtypes = [vp, i32, dp, dp]
        L.spgx_vbd_reset.argtypes = [vp]
        L.spgx_vbd_residual.argtypes = [vp, dp]
        L.spgx_vbd_num_colors.argtypes = [vp, i32, ip]
        L.spgx_vbd_get_colors.argtypes = [vp, i32, ip]
        L.spgx_vbd_get_adjacency.argtypes = [vp, i32, ip, ip, C.POINTER(C.c_int64)]
        L.spgx_vbd_get_launch.argtypes = [vp, ip, ip, ip]
        L.spgx_vbd_set_picks.argtypes = [vp, i32, ip, ip, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.spgx_vbd_test_stall_tile.argtypes = [vp, i32]
        L.spgx_vbd_set_warm_start_smoothing.argtypes = [vp, i32]
        L.spgx_vbd_profile_sweeps.argtypes = [vp, i32, dp]
        L.spgx_eval_vertex_blocks.argtypes = [i32, i32, dp, dp, ip, dp, dp]
        L.spgx_eval_constraints.argtypes = [i32, i32, dp, dp, dp, dp]
        L.spgx_eval_vertex_blocks_noalloc.argtypes = [i32, i32, dp, dp, ip, dp, dp]
        L.spgx_xpbd_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(XpbdParams), C.POINTER(vp)]
        L.spgx_xpbd_destroy.argtypes = [vp]
        L.spgx_xpbd_set_params.argtypes = [vp, C.POINTER(XpbdParams)]
        L.spgx_xpbd_step.argtypes = [vp, C.POINTER(StepStats)]
        L.spgx_xpbd_get_state.argtypes = [vp, i32, dp, dp]
        L.spgx_xpbd_set_state.argtypes = [vp, i32, dp, dp]
        L.spgx_xpbd_reset.argtypes = [vp]
        L.spgx_xpbd_get_stencil_colors.argtypes = [vp, i32, i32, ip]
        L.spgx_xpbd_test_stall.argtypes = [vp]
        L.spgx_color_vertices.argtypes = [C.POINTER(ObjectDesc), ip]
        L.spgx_color_stencils.argtypes = [C.POINTER(EnergyDesc), ip]
        L.spgx_incidences.argtypes = [C.POINTER(ObjectDesc), ip, ip, C.POINTER(C.c_int64)]
        L.spgx_incidences_device.argtypes = [C.POINTER(ObjectDesc), i32, ip, ip, C.POINTER(C.c_int64)]
        L.spgx_material_count.restype = i32
        L.spgx_material_count.argtypes = [i32]
        L.spgx_precompute_params.argtypes = [i32, i32, ip, i32, C.POINTER(C.c_double), C.POINTER(C.c_double), i32,
                                             C.POINTER(C.c_double), i32]
        L.spgx_precompute_params_host.argtypes = [i32, i32, ip, i32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                  i32, C.POINTER(C.c_double)]
        fp = C.POINTER(C.c_float)
        L.spgx_mlp_num_params.restype = i32
        L.spgx_mlp_create.argtypes = [C.c_uint64, i32, C.POINTER(vp)]
        L.spgx_mlp_destroy.argtypes = [vp]
        L.spgx_mlp_get_weights.argtypes = [vp, fp]
        L.spgx_mlp_set_weights.argtypes = [vp, fp]
        L.spgx_mlp_forward.argtypes = [vp, i32, fp, fp]
        L.spgx_mlp_loss_grad.argtypes = [vp, i32, fp, fp, fp, fp]
        L.spgx_mlp_train.argtypes = [vp, i32, fp, fp, i32, i32, C.c_float, C.c_uint64, fp]
        L.spgx_vbd_set_warm_start.argtypes = [vp, vp, i32]
        L.spgx_vbd_step_record.argtypes = [vp, fp, fp, C.POINTER(StepStats)]
        L.spgx_vbd_get_vertex_order.argtypes = [vp, ip]
        L.spgx_implicit_params_default.argtypes = [C.POINTER(ImplicitParams)]
        L.spgx_implicit_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(ImplicitParams), C.POINTER(vp)]
        L.spgx_implicit_destroy.argtypes = [vp]
        L.spgx_implicit_step.argtypes = [vp, C.POINTER(StepStats)]
        L.spgx_implicit_get_state.argtypes = [vp, i32, dp, dp]
        L.spgx_implicit_set_state.argtypes = [vp, i32, dp, dp]
        L.spgx_implicit_reset.argtypes = [vp]
        L.spgx_implicit_get_step_size.argtypes = [vp, dp]
        L.spgx_implicit_test_stall.argtypes = [vp]
        L.spgx_implicit_set_params.argtypes = [vp, C.POINTER(ImplicitParams)]
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise SpgxError(status, lib().spgx_last_error_string().decode())


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Descriptor:
    """spgx_scene_desc over a list of objects exposing x, mass, energies (type, stencils,
    params) and optionally v; keeps the numpy buffers alive."""

    def __init__(self, objects):
        self.keep = []
        objs = (ObjectDesc * max(1, len(objects)))()
        for k, ob in enumerate(objects):
            x = np.ascontiguousarray(ob.x, dtype=np.float64).reshape(-1)
            m = np.ascontiguousarray(ob.mass, dtype=np.float64).reshape(-1)
            v = getattr(ob, "v", None)
            v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
            es = (EnergyDesc * max(1, len(ob.energies)))()
            for i, e in enumerate(ob.energies):
                st = np.ascontiguousarray(e.stencils, dtype=np.int32).reshape(-1)
                pa = np.ascontiguousarray(e.params, dtype=np.float64).reshape(-1)
                n = len(st) // STENCIL_SIZE[e.type] if e.type in STENCIL_SIZE else 0
                self.keep += [st, pa]
                es[i] = EnergyDesc(e.type, n, _p(st, C.c_int32), _p(pa, C.c_double))
            self.keep += [x, m, v, es]
            objs[k] = ObjectDesc(len(m), _p(x, C.c_double), None if v is None else _p(v, C.c_double),
                                 _p(m, C.c_double), len(ob.energies), es)
        self.keep.append(objs)
        self.scene = SceneDesc(len(objects), objs)


def vbd_params(dt=0.01, substeps=1, iterations=1, gravity=(0.0, -9.8, 0.0), tolerance=0.0, max_iterations=1000,
               check_interval=10, fallback_condition=1e6, lanes_per_vertex=0, block_size=0, use_graph=1,
               device=0, kernel=0, tile_vertices=0) -> VbdParams:
    p = VbdParams()
    lib().spgx_vbd_params_default(C.byref(p))
    p.dt, p.substeps, p.iterations = dt, substeps, iterations
    p.gravity = (C.c_double * 3)(*gravity)
    p.tolerance, p.max_iterations, p.check_interval = tolerance, max_iterations, check_interval
    p.fallback_condition = fallback_condition
    p.lanes_per_vertex, p.block_size, p.use_graph, p.device = lanes_per_vertex, block_size, use_graph, device
    p.kernel, p.tile_vertices = kernel, tile_vertices
    return p


class VbdSolver:
    """GB300 VBD over a list of objects (one handle, one CUDA stream)."""

    def __init__(self, objects, **params):
        self.objects_nv = [len(np.asarray(o.mass).reshape(-1)) for o in objects]
        self.n_energies = [len(o.energies) for o in objects]
        self._d = Descriptor(objects)
        self.params = vbd_params(**params)
        h = C.c_void_p()
        check(lib().spgx_vbd_create(C.byref(self._d.scene), C.byref(self.params), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().spgx_vbd_destroy(self.h)
            self.h = None

    __del__ = close

    def set_params(self, **changes):
        for k, v in changes.items():
            if k == "gravity":
                self.params.gravity = (C.c_double * 3)(*v)
            else:
                setattr(self.params, k, v)
        check(lib().spgx_vbd_set_params(self.h, C.byref(self.params)))

    def step(self) -> StepStats:
        st = StepStats()
        check(lib().spgx_vbd_step(self.h, C.byref(st)))
        return st

    def state(self, obj=0):
        n = self.objects_nv[obj]
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        check(lib().spgx_vbd_get_state(self.h, obj, _p(x, C.c_double), _p(v, C.c_double)))
        return x, v

    def get_state_into(self, obj, x, v=None):
        check(lib().spgx_vbd_get_state(self.h, obj, _p(x, C.c_double), None if v is None else _p(v, C.c_double)))

    def set_state(self, obj, x, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        check(lib().spgx_vbd_set_state(self.h, obj, _p(x, C.c_double), None if vv is None else _p(vv, C.c_double)))

    def reset(self):
        check(lib().spgx_vbd_reset(self.h))

    def residual(self) -> float:
        r = C.c_double()
        check(lib().spgx_vbd_residual(self.h, C.byref(r)))
        return r.value

    def colors(self, obj=0):
        c = np.zeros(self.objects_nv[obj], np.int32)
        check(lib().spgx_vbd_get_colors(self.h, obj, _p(c, C.c_int32)))
        return c

    def n_colors(self, obj=0):
        n = C.c_int32()
        check(lib().spgx_vbd_num_colors(self.h, obj, C.byref(n)))
        return n.value

    def adjacency(self, obj=0):
        tot = C.c_int64()
        check(lib().spgx_vbd_get_adjacency(self.h, obj, None, None, C.byref(tot)))
        counts = np.zeros(self.objects_nv[obj] * self.n_energies[obj], np.int32)
        ent = np.zeros((max(1, tot.value), 2), np.int32)
        check(lib().spgx_vbd_get_adjacency(self.h, obj, _p(counts, C.c_int32), _p(ent, C.c_int32), C.byref(tot)))
        return counts.reshape(self.objects_nv[obj], self.n_energies[obj]), ent[:tot.value]

    def profile_sweeps(self, iterations=3):
        """Mean CUDA-event duration (ms) of each colour launch over `iterations` sweeps."""
        n = C.c_int32()
        check(lib().spgx_vbd_num_colors(self.h, -1, C.byref(n)))
        out = np.zeros(n.value)
        check(lib().spgx_vbd_profile_sweeps(self.h, iterations, _p(out, C.c_double)))
        return out

    def set_warm_start(self, mlp=None, mode=None):
        """Initial guess of every substep: mode 0 inertial (history kept), 1 learned (`mlp`, an
        Mlp), 2 extrapolated acceleration. Default: 1 with an mlp, else 0."""
        if mode is None:
            mode = 0 if mlp is None else 1
        self._mlp = mlp
        check(lib().spgx_vbd_set_warm_start(self.h, None if mlp is None else mlp.h, int(mode)))

    def step_record(self):
        """One step returning (stats, features [n x 24], targets [n x 3]) in internal vertex order."""
        n = sum(self.objects_nv)
        f = np.zeros((n, WARM_FEATURES), np.float32)
        t = np.zeros((n, 3), np.float32)
        st = StepStats()
        check(lib().spgx_vbd_step_record(self.h, _p(f, C.c_float), _p(t, C.c_float), C.byref(st)))
        return st, f, t

    def vertex_order(self) -> np.ndarray:
        """ext_of_internal: scene vertex index (objects concatenated) of each internal row."""
        out = np.zeros(sum(self.objects_nv), np.int32)
        check(lib().spgx_vbd_get_vertex_order(self.h, _p(out, C.c_int32)))
        return out

    def set_picks(self, picks):
        """Dynamic anchors for picking: a list of (object, vertex, target xyz, stiffness)."""
        n = len(picks)
        o = np.array([p[0] for p in picks], np.int32).reshape(-1)
        v = np.array([p[1] for p in picks], np.int32).reshape(-1)
        t = np.array([p[2] for p in picks], np.float64).reshape(-1)
        k = np.array([p[3] for p in picks], np.float64).reshape(-1)
        o, v, t, k = (np.ascontiguousarray(a) for a in (o, v, t, k))
        check(lib().spgx_vbd_set_picks(self.h, n, _p(o, C.c_int32), _p(v, C.c_int32), _p(t, C.c_double),
                                       _p(k, C.c_double)))

    def set_warm_start_smoothing(self, passes):
        """One-ring smoothing passes over the network's correction before the learned guess."""
        check(lib().spgx_vbd_set_warm_start_smoothing(self.h, passes))

    def test_stall_tile(self, tile):
        """Failure-detection test hook: the next dataflow step's waits on `tile` run out."""
        check(lib().spgx_vbd_test_stall_tile(self.h, tile))

    def launch(self):
        """(kernel, lanes_per_vertex or tile vertices, block size) chosen by the solver."""
        k, g, b = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().spgx_vbd_get_launch(self.h, C.byref(k), C.byref(g), C.byref(b)))
        return k.value, g.value, b.value


WARM_FEATURES = 24


class Mlp:
    """The warm-start network (24 -> 128 -> 128 -> 128 -> 3, GELU) on one GPU."""

    def __init__(self, seed=0, device=0, weights=None):
        h = C.c_void_p()
        check(lib().spgx_mlp_create(seed, device, C.byref(h)))
        self.h = h
        if weights is not None:
            self.set_weights(weights)

    @staticmethod
    def num_params() -> int:
        return lib().spgx_mlp_num_params()

    def close(self):
        if getattr(self, "h", None):
            lib().spgx_mlp_destroy(self.h)
            self.h = None

    __del__ = close

    def weights(self) -> np.ndarray:
        w = np.zeros(self.num_params(), np.float32)
        check(lib().spgx_mlp_get_weights(self.h, _p(w, C.c_float)))
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32).reshape(-1)
        if w.size != self.num_params():
            raise ValueError(f"expected {self.num_params()} weights, got {w.size}")
        check(lib().spgx_mlp_set_weights(self.h, _p(w, C.c_float)))

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, WARM_FEATURES)
        y = np.zeros((x.shape[0], 3), np.float32)
        check(lib().spgx_mlp_forward(self.h, x.shape[0], _p(x, C.c_float), _p(y, C.c_float)))
        return y

    def loss_grad(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, WARM_FEATURES)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1, 3)
        g = np.zeros(self.num_params(), np.float32)
        loss = C.c_float()
        check(lib().spgx_mlp_loss_grad(self.h, x.shape[0], _p(x, C.c_float), _p(y, C.c_float), C.byref(loss),
                                       _p(g, C.c_float)))
        return loss.value, g

    def train(self, x, y, steps, batch=4096, lr=1e-3, seed=0) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, WARM_FEATURES)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1, 3)
        loss = C.c_float()
        check(lib().spgx_mlp_train(self.h, x.shape[0], _p(x, C.c_float), _p(y, C.c_float), steps, batch, lr, seed,
                                   C.byref(loss)))
        return loss.value


(NEWTON_DX, NEWTON_DV, NEWTON_ROBUST, BARAFF_WITKIN, BDF2, STATIC_NEWTON, QUASI_STATIC_NEWTON,
 QUASI_STATIC_NEWTON_ROBUST, SYMPLECTIC_EULER) = range(9)


class ImplicitSolver:
    """The reference's global solvers on one GPU: `method` is one of NEWTON_DX (default),
    NEWTON_DV, NEWTON_ROBUST, BARAFF_WITKIN, BDF2, STATIC_NEWTON, QUASI_STATIC_NEWTON,
    QUASI_STATIC_NEWTON_ROBUST and SYMPLECTIC_EULER."""

    def __init__(self, objects, dt=0.01, substeps=1, gravity=(0.0, -9.8, 0.0), cg_threshold=1e-5,
                 cg_max_iterations=300, device=0, method=NEWTON_DX, cg_precision=0):
        self.objects_nv = [len(np.asarray(o.mass).reshape(-1)) for o in objects]
        self._d = Descriptor(objects)
        p = ImplicitParams()
        lib().spgx_implicit_params_default(C.byref(p))
        p.dt, p.substeps = dt, substeps
        p.gravity = (C.c_double * 3)(*gravity)
        p.cg_threshold, p.cg_max_iterations, p.device = cg_threshold, cg_max_iterations, device
        p.method, p.cg_precision = method, cg_precision
        self.params = p
        h = C.c_void_p()
        check(lib().spgx_implicit_create(C.byref(self._d.scene), C.byref(p), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().spgx_implicit_destroy(self.h)
            self.h = None

    __del__ = close

    def step(self) -> StepStats:
        st = StepStats()
        check(lib().spgx_implicit_step(self.h, C.byref(st)))
        return st

    def state(self, obj=0):
        n = self.objects_nv[obj]
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        check(lib().spgx_implicit_get_state(self.h, obj, _p(x, C.c_double), _p(v, C.c_double)))
        return x, v

    def set_state(self, obj, x, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        check(lib().spgx_implicit_set_state(self.h, obj, _p(x, C.c_double), None if vv is None else _p(vv, C.c_double)))

    def reset(self):
        check(lib().spgx_implicit_reset(self.h))

    def set_params(self, dt=None, substeps=None, gravity=None):
        """Changes dt / substeps / gravity for the following steps; the step control and
        BDF2's history carry over."""
        p = self.params
        if dt is not None:
            p.dt = dt
        if substeps is not None:
            p.substeps = substeps
        if gravity is not None:
            p.gravity = (C.c_double * 3)(*gravity)
        check(lib().spgx_implicit_set_params(self.h, C.byref(p)))

    def step_size(self) -> float:
        """The robust methods' current substep (-1 before the first step)."""
        d = C.c_double()
        check(lib().spgx_implicit_get_step_size(self.h, C.byref(d)))
        return d.value

    def test_stall(self):
        """Failure-detection test hook: the next CG solve's bounded barrier waits run out."""
        check(lib().spgx_implicit_test_stall(self.h))


class XpbdSolver:
    def __init__(self, objects, dt=0.01, substeps=1, gravity=(0.0, -9.8, 0.0), block_size=0, use_graph=1, device=0,
                 kernel=0):
        self.objects_nv = [len(np.asarray(o.mass).reshape(-1)) for o in objects]
        self.n_stencils = [[len(np.asarray(e.stencils).reshape(-1)) // STENCIL_SIZE[e.type] for e in o.energies]
                           for o in objects]
        self._d = Descriptor(objects)
        p = XpbdParams()
        lib().spgx_xpbd_params_default(C.byref(p))
        p.dt, p.substeps = dt, substeps
        p.gravity = (C.c_double * 3)(*gravity)
        p.block_size, p.use_graph, p.device, p.kernel = block_size, use_graph, device, kernel
        self.params = p
        h = C.c_void_p()
        check(lib().spgx_xpbd_create(C.byref(self._d.scene), C.byref(p), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().spgx_xpbd_destroy(self.h)
            self.h = None

    __del__ = close

    def step(self) -> StepStats:
        st = StepStats()
        check(lib().spgx_xpbd_step(self.h, C.byref(st)))
        return st

    def state(self, obj=0):
        n = self.objects_nv[obj]
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        check(lib().spgx_xpbd_get_state(self.h, obj, _p(x, C.c_double), _p(v, C.c_double)))
        return x, v

    def get_state_into(self, obj, x, v=None):
        check(lib().spgx_xpbd_get_state(self.h, obj, _p(x, C.c_double), None if v is None else _p(v, C.c_double)))

    def set_state(self, obj, x, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        check(lib().spgx_xpbd_set_state(self.h, obj, _p(x, C.c_double), None if vv is None else _p(vv, C.c_double)))

    def test_stall(self):
        """Failure-detection test hook: the next persistent step's bounded waits run out."""
        check(lib().spgx_xpbd_test_stall(self.h))

    def stencil_colors(self, obj, energy):
        out = np.zeros(self.n_stencils[obj][energy], np.int32)
        check(lib().spgx_xpbd_get_stencil_colors(self.h, obj, energy, _p(out, C.c_int32)))
        return out


def eval_vertex_blocks(etype, X, params, slots):
    """GPU FP32 gradient segments (n, 3) and Hessian blocks (n, 3, 3) of n incidences."""
    S, P = STENCIL_SIZE[etype], PARAM_COUNT[etype]
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, S * 3)
    n = X.shape[0]
    prm = np.ascontiguousarray(params, dtype=np.float64).reshape(n, P)
    sl = np.ascontiguousarray(slots, dtype=np.int32).reshape(n)
    g = np.zeros((n, 3))
    H = np.zeros((n, 9))
    check(lib().spgx_eval_vertex_blocks(etype, n, _p(X, C.c_double), _p(prm, C.c_double), _p(sl, C.c_int32),
                                        _p(g, C.c_double), _p(H, C.c_double)))
    return g, H.reshape(n, 3, 3)


def eval_vertex_blocks_noalloc(etype, X, params, slots):
    """Same as eval_vertex_blocks through the allocation-free entry point (n <= 4096)."""
    S, P = STENCIL_SIZE[etype], PARAM_COUNT[etype]
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, S * 3)
    n = X.shape[0]
    prm = np.ascontiguousarray(params, dtype=np.float64).reshape(n, P)
    sl = np.ascontiguousarray(slots, dtype=np.int32).reshape(n)
    g = np.zeros((n, 3))
    H = np.zeros((n, 9))
    check(lib().spgx_eval_vertex_blocks_noalloc(etype, n, _p(X, C.c_double), _p(prm, C.c_double),
                                                _p(sl, C.c_int32), _p(g, C.c_double), _p(H, C.c_double)))
    return g, H.reshape(n, 3, 3)


def eval_constraints(etype, X, params):
    S, P = STENCIL_SIZE[etype], PARAM_COUNT[etype]
    nc = lib().spgx_num_constraints(etype)
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, S * 3)
    n = X.shape[0]
    prm = np.ascontiguousarray(params, dtype=np.float64).reshape(n, P)
    c = np.zeros((n, nc))
    g = np.zeros((n, nc, 3 * S))
    check(lib().spgx_eval_constraints(etype, n, _p(X, C.c_double), _p(prm, C.c_double), _p(c, C.c_double),
                                      _p(g, C.c_double)))
    return c, g


def color_vertices(obj) -> np.ndarray:
    """Host-side greedy vertex colouring of one object (no device needed)."""
    d = Descriptor([obj])
    out = np.zeros(max(1, d.scene.objects[0].n_vertices), np.int32)
    check(lib().spgx_color_vertices(C.byref(d.scene.objects[0]), _p(out, C.c_int32)))
    return out[:d.scene.objects[0].n_vertices]


def color_stencils(energy) -> np.ndarray:
    st = np.ascontiguousarray(energy.stencils, dtype=np.int32).reshape(-1)
    pa = np.ascontiguousarray(energy.params, dtype=np.float64).reshape(-1)
    n = len(st) // STENCIL_SIZE[energy.type]
    e = EnergyDesc(energy.type, n, _p(st, C.c_int32), _p(pa, C.c_double))
    out = np.zeros(max(1, n), np.int32)
    check(lib().spgx_color_stencils(C.byref(e), _p(out, C.c_int32)))
    return out[:n]


def incidences(obj, device=None):
    """Reference-order incidence lists: counts (V, n_energies) and (stencil, slot) pairs,
    computed on the host, or on the GPU `device` when given."""
    d = Descriptor([obj])
    ob = d.scene.objects[0]
    tot = C.c_int64()
    if device is None:
        fn = lambda c, e: lib().spgx_incidences(C.byref(ob), c, e, C.byref(tot))  # noqa: E731
    else:
        fn = lambda c, e: lib().spgx_incidences_device(C.byref(ob), device, c, e, C.byref(tot))  # noqa: E731
    check(fn(None, None))
    counts = np.zeros(max(1, ob.n_vertices * ob.n_energies), np.int32)
    ent = np.zeros((max(1, tot.value), 2), np.int32)
    check(fn(_p(counts, C.c_int32), _p(ent, C.c_int32)))
    return counts[:ob.n_vertices * ob.n_energies].reshape(ob.n_vertices, ob.n_energies), ent[:tot.value]


def precompute_params(etype, stencils, x0, material, device=0):
    """The energy's addStencil + preparePrecomputations on the GPU `device` (None: on the host
    through the host energy classes): packed params (n, P) from the rest positions and the
    per-stencil material values (one row, or one per stencil)."""
    st = np.ascontiguousarray(stencils, np.int32).reshape(-1, STENCIL_SIZE[etype])
    x0 = np.ascontiguousarray(x0, np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(material, np.float64)
    M = lib().spgx_material_count(etype)
    stride = 0 if m.ndim == 1 else M
    m = m.reshape(-1, M)
    out = np.zeros((len(st), PARAM_COUNT[etype]))
    args = (etype, len(st), _p(st, C.c_int32), len(x0), _p(x0, C.c_double), _p(m, C.c_double), stride,
            _p(out, C.c_double))
    if device is None:
        check(lib().spgx_precompute_params_host(*args))
    else:
        check(lib().spgx_precompute_params(*args, device))
    return out
