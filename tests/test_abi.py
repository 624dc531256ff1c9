"""The C ABI library loads and exports every entry point its headers declare; calls that
need a device fail cleanly without one."""
import ctypes as C
import os
import re

import pytest

from spg_gb300 import native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in ("spgx.h", "spgx_scenes.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            text = f.read()
        names |= set(re.findall(r"\b(spgx_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    names = _declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_sizes_and_defaults():
    lib = N.lib()
    assert lib.spgx_api_version() == 1
    for t in (N.SPRING, N.ANCHOR, N.BENDING, N.STVK, N.SNH):
        assert lib.spgx_stencil_size(t) == N.STENCIL_SIZE[t]
        assert lib.spgx_param_count(t) == N.PARAM_COUNT[t]
    assert lib.spgx_stencil_size(42) == 0
    p = N.vbd_params()
    assert p.fallback_condition == 1e6 and p.use_graph == 1 and p.tile_vertices == 0


def _has_device():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False


@pytest.mark.skipif(_has_device(), reason="checks the behaviour without a device")
def test_no_device_errors_cleanly():
    from tests import scenes
    obj = scenes.cloth_cfg1(5)
    with pytest.raises(N.SpgxError) as e:
        N.VbdSolver([obj], dt=1 / 60)
    assert e.value.status in (3, 6)
    with pytest.raises(N.SpgxError):
        N.eval_vertex_blocks(N.SPRING, [[0, 0, 0, 1, 0, 0]], [[1, 1, 1]], [0])


def test_invalid_arguments_rejected_before_device_use():
    lib = N.lib()
    h = C.c_void_p()
    assert lib.spgx_vbd_create(None, None, C.byref(h)) != 0
    assert lib.spgx_vbd_step(None, None) == 1
    assert lib.spgx_xpbd_step(None, None) == 1
    assert b"NULL" in lib.spgx_last_error_string()
