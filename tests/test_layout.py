"""Host-side setup of the shipped library (no device): bit-exact greedy colouring and
incidence lists against the oracle, the reference's compiled colouring and the golden
fixtures; scene builders bit-exact with the oracle's; input validation."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from spg_gb300 import native as N
from spg_gb300 import scenes as S
from tests import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "coloring_golden.json")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def _same_object(a, b):
    assert a.nv == b.nv
    assert np.array_equal(a.x, b.x) and np.array_equal(a.mass, b.mass) and np.array_equal(a.x0, b.x0)
    assert [e.type for e in a.energies] == [e.type for e in b.energies]
    for ea, eb in zip(a.energies, b.energies):
        assert np.array_equal(ea.stencils, eb.stencils)
        assert np.array_equal(ea.params, eb.params)


def test_scene_builders_bit_exact_with_oracle():
    _same_object(S.cloth(33).objects[0], scenes.cloth_cfg1(33))
    _same_object(S.tet_beam().objects[0], scenes.beam_cfg2())
    sx, sy, sz = 0.025 * 8, 0.025 * 3, 0.025 * 3
    _same_object(S.tet_beam(9, 4, 4, split=5).objects[0],
                 O.build_tet_beam(1000.0 * sx * sy * sz, sx, sy, sz, 9, 4, 4, 1e6, 0.45, 1e4, 5))
    _same_object(S.spring_cloth(129).objects[0], scenes.spring_cloth_cfg3(129))
    for a, b in zip(S.patch_batch(12, 16, 40, seed=5).objects, scenes.patch_batch_cfg4(12, 16, 40, seed=5)):
        _same_object(a, b)


def test_colouring_and_incidences_match_oracle():
    for obj in (scenes.cloth_cfg1(33), scenes.beam_cfg2(9, 5, 5), scenes.spring_cloth_cfg3(65),
                *scenes.patch_batch_cfg4(4, 8, 24, seed=1)):
        ref = O.Vbd(obj, 1 / 60, 1, 1, scenes.GRAVITY)
        assert np.array_equal(N.color_vertices(obj), ref.colors())
        c1, e1 = N.incidences(obj)
        c2, e2 = ref.adjacency(len(obj.energies))
        assert np.array_equal(c1, c2) and np.array_equal(e1, e2)
        x = O.Xpbd(obj, 1 / 60, 1, scenes.GRAVITY)
        for k, e in enumerate(obj.energies):
            assert np.array_equal(N.color_stencils(e), x.stencil_colors(k))


def test_colouring_matches_reference_golden_at_full_size():
    with open(GOLDEN) as f:
        g = json.load(f)["scenes"]
    cloth = S.spring_cloth(513).objects[0]
    assert _digest(N.color_vertices(cloth)) == g["spring_cloth_513"]["sha256"]
    for k, e in enumerate(cloth.energies):
        assert _digest(N.color_stencils(e)) == g["spring_cloth_513"]["stencil_colors"][k]["sha256"]
    beam = S.tet_beam().objects[0]
    assert _digest(N.color_vertices(beam)) == g["beam_41x11x11_6tet"]["sha256"]
    assert N.color_vertices(S.cloth(33).objects[0]).tolist() == g["cloth_33"]["colors"]
    for o, gg in zip(S.patch_batch(8, 16, 128, seed=2024).objects, g["patch_batch_8"]):
        assert _digest(N.color_vertices(o)) == gg["sha256"]


@pytest.mark.skipif(O.ref_lib() is None, reason="reference checkout not present")
def test_colouring_equals_compiled_reference_on_edge_cases():
    E = O.Energy
    cases = [
        # isolated vertices, anchors only, a repeated index inside a stencil
        O.SceneObject(np.zeros((5, 3)), np.ones(5), [E(O.ANCHOR, np.array([[0], [3]], np.int32), np.zeros((2, 5)))]),
        O.SceneObject(np.zeros((4, 3)), np.ones(4), [E(O.SPRING, np.array([[2, 2], [0, 3], [3, 1]], np.int32),
                                                       np.ones((3, 3)))]),
        O.SceneObject(np.zeros((1, 3)), np.ones(1), []),
    ]
    for obj in cases:
        assert np.array_equal(N.color_vertices(obj), O.ref_color_vertices(obj))
        for e in obj.energies:
            assert np.array_equal(N.color_stencils(e), O.ref_color_stencils(e))


def test_validation_errors():
    E = O.Energy
    bad_index = O.SceneObject(np.zeros((3, 3)), np.ones(3), [E(O.SPRING, np.array([[0, 3]], np.int32), np.ones((1, 3)))])
    with pytest.raises(N.SpgxError, match="invalid vertex"):
        N.color_vertices(bad_index)
    bad_type = O.SceneObject(np.zeros((3, 3)), np.ones(3), [E(99, np.array([[0, 1]], np.int32), np.ones((1, 3)))])
    with pytest.raises(N.SpgxError):
        N.color_vertices(bad_type)
    with pytest.raises(N.SpgxError):
        S.cloth(3, anchors=[100])


def test_empty_object():
    obj = O.SceneObject(np.zeros((0, 3)), np.zeros(0), [])
    assert N.color_vertices(obj).size == 0
    counts, ent = N.incidences(obj)
    assert counts.size == 0 and ent.size == 0
