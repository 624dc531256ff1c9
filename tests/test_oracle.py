"""The FP64 oracle: derivatives three ways (its AD in the reference's full-element form, its
vertex-restricted AD, central differences), known answers, and its literal colouring against
the reference's own compiled colouring and the committed golden fixtures."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "coloring_golden.json")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def _samples(obj, n, rng, scale):
    for e in obj.energies:
        for i in rng.integers(0, e.n, size=min(n, e.n)):
            X = obj.x[e.stencils[i]] + rng.normal(scale=scale, size=(e.stencils.shape[1], 3))
            yield e.type, X, e.params[i]


@pytest.mark.parametrize("which", ["cloth", "beam", "springs"])
def test_ad_block_equals_full_element_ad_and_finite_differences(which):
    rng = np.random.default_rng(1)
    obj = {"cloth": lambda: scenes.cloth_cfg1(9), "beam": lambda: scenes.beam_cfg2(5, 3, 3),
           "springs": lambda: scenes.spring_cloth_cfg3(9)}[which]()
    scale = 0.05 * float(np.ptp(obj.x0, axis=0).max()) / 8
    for etype, X, p in _samples(obj, 15, rng, scale):
        for slot in range(X.shape[0]):
            gF, HF = O.element_block(etype, X, p, slot, O.FULL_AD)
            gV, HV = O.element_block(etype, X, p, slot, O.VERTEX_AD)
            assert np.allclose(gF, gV, rtol=1e-11, atol=1e-13 * max(1, np.abs(gF).max()))
            assert np.allclose(HF, HV, rtol=1e-11, atol=1e-13 * max(1, np.abs(HF).max()))
            h = 1e-6 * max(1e-3, np.abs(X).max())
            gfd, Hfd = np.zeros(3), np.zeros((3, 3))
            for a in range(3):
                Xp, Xm = X.copy(), X.copy()
                Xp[slot, a] += h
                Xm[slot, a] -= h
                gfd[a] = (O.element_energy(etype, Xp, p) - O.element_energy(etype, Xm, p)) / (2 * h)
                gp, _ = O.element_block(etype, Xp, p, slot, O.FULL_AD)
                gm, _ = O.element_block(etype, Xm, p, slot, O.FULL_AD)
                Hfd[:, a] = (gp - gm) / (2 * h)
            assert np.abs(gF - gfd).max() <= 1e-5 * max(np.abs(gF).max(), 1e-12) + 1e-9
            assert np.abs(HF - Hfd).max() <= 1e-5 * max(np.abs(HF).max(), 1e-12) + 1e-9


@pytest.mark.parametrize("which", ["cloth", "beam", "springs"])
def test_zero_gradient_at_rest(which):
    obj = {"cloth": lambda: scenes.cloth_cfg1(9), "beam": lambda: scenes.beam_cfg2(5, 3, 3),
           "springs": lambda: scenes.spring_cloth_cfg3(9)}[which]()
    for e in obj.energies:
        for i in range(e.n):
            X = obj.x0[e.stencils[i]] if e.type != O.ANCHOR else np.array([e.params[i][:3]])
            for slot in range(X.shape[0]):
                g, _ = O.element_block(e.type, X, e.params[i], slot, O.FULL_AD)
                assert np.abs(g).max() <= 1e-9 * max(1.0, np.abs(e.params[i]).max())


def test_energy_viewer_known_answers():
    """One-element scenes of apps/energyViewer.cpp:20-30 and :125-137 with closed-form values."""
    # StVK triangle (0,0,0),(1,0,0),(0,1,0), young 1, poisson 0: rest area 1/2, K = diag(1,1,1/2)/2.
    tri = O.build_cloth(1.0, 1.0, 1.0, 2, 2, 1.0, 0.0, 1.0, 1.0, True, anchors=[])
    stvk = next(e for e in tri.energies if e.type == O.STVK)
    st, p = stvk.stencils[0], stvk.params[0]
    X = tri.x0[st].copy()
    s = 1.3
    X[:, 0] *= s  # uniform stretch along x: F = diag(s, 1), E00 = (s^2 - 1) / 2
    area = 0.5
    e00 = 0.5 * (s * s - 1)
    expected = 0.5 * area * 1.0 * e00 * e00
    assert abs(O.element_energy(O.STVK, X, p) - expected) <= 1e-14
    # SNH unit tet, young 10, poisson 0.2: mu = 10/2.4, lambda = mu/0.6, alpha = 1 + mu/lambda.
    beam = O.build_tet_beam(1.0, 1.0, 1.0, 1.0, 2, 2, 2, 10.0, 0.2, 1.0, 6)
    snh = next(e for e in beam.energies if e.type == O.SNH)
    mu = 10 / (2 * 1.2)
    lam = mu / (1 - 0.4)
    alpha = 1 + mu / lam
    vol = 1.0 / 6.0
    assert np.isclose(snh.params[0][11], alpha)
    assert np.isclose(snh.params[0][9], lam * vol) and np.isclose(snh.params[0][10], mu * vol)
    # At rest F = I: E = 1/2 lambda (1 - alpha)^2 with the volume-scaled lambda.
    Xr = beam.x0[snh.stencils[0]]
    assert abs(O.element_energy(O.SNH, Xr, snh.params[0]) - 0.5 * lam * vol * (1 - alpha) ** 2) <= 1e-12
    # Spring of rest length 1 stretched to 1.5 with k = 2: E = 1/2 k 0.25, |g| = k 0.5.
    p_s = np.array([1.0, 2.0, 0.5])
    Xs = np.array([[0.0, 0, 0], [1.5, 0, 0]])
    assert abs(O.element_energy(O.SPRING, Xs, p_s) - 0.25) <= 1e-15
    g, H = O.element_block(O.SPRING, Xs, p_s, 0, O.FULL_AD)
    assert np.allclose(g, [-1.0, 0, 0]) and np.allclose(np.diag(H), [2.0, 2 * (1 - 1 / 1.5), 2 * (1 - 1 / 1.5)])
    # Bending of a flat hinge folded by 90 degrees: theta = -pi/2 with the reference's sign.
    pb = np.array([0.0, 1.0, 1.0])
    Xb = np.array([[0.0, 0, 0], [1.0, 0, 0], [0.5, 1, 0], [0.5, 0, 1.0]])
    c, _ = O.element_constraints(O.BENDING, Xb, pb)
    assert np.isclose(abs(c[0]), np.pi / 2)


def test_constraint_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    for obj in (scenes.cloth_cfg1(9), scenes.beam_cfg2(5, 3, 3), scenes.spring_cloth_cfg3(9)):
        for etype, X, p in _samples(obj, 10, rng, 0.01):
            c, G = O.element_constraints(etype, X, p)
            h = 1e-7
            flat = X.reshape(-1)
            for d in range(flat.size):
                xp, xm = flat.copy(), flat.copy()
                xp[d] += h
                xm[d] -= h
                cp, _ = O.element_constraints(etype, xp.reshape(X.shape), p)
                cm, _ = O.element_constraints(etype, xm.reshape(X.shape), p)
                fd = (cp - cm) / (2 * h)
                assert np.allclose(G[:, d], fd, rtol=1e-5, atol=1e-6 * max(1, np.abs(G).max()))


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)["scenes"]


def test_literal_colouring_matches_reference_golden(golden):
    cases = {"cloth_33": scenes.cloth_cfg1(33), "spring_cloth_65": scenes.spring_cloth_cfg3(65),
             "beam_9x4x4_5tet": O.build_tet_beam(62.5, 0.2, 0.075, 0.075, 9, 4, 4, 1e6, 0.45, 1e4, 5),
             "beam_41x11x11_6tet": scenes.beam_cfg2()}
    for name, obj in cases.items():
        g = golden[name]
        colors = O.color_vertices(obj)
        assert _digest(colors) == g["sha256"], name
        assert np.bincount(colors).tolist() == g["histogram"]
        if "colors" in g:
            assert colors.tolist() == g["colors"]
        s = O.Vbd(obj, 1 / 60, 1, 1, scenes.GRAVITY)
        for k, e in enumerate(obj.energies):
            assert _digest(O.Xpbd(obj, 1 / 60, 1, scenes.GRAVITY).stencil_colors(k)) == g["stencil_colors"][k]["sha256"]
        del s


def test_scene_counts_of_the_benchmark_scenes(golden):
    """Vertex, incidence, colour and stencil counts of the 33^2 StVK cloth, the 41x11x11 six-tet
    bar and the 513^2 spring cloth, as the reference's scene builders give them."""
    g1, g2, g3 = golden["cloth_33"], golden["beam_41x11x11_6tet"], golden["spring_cloth_513"]
    assert (g1["n_vertices"], g1["n_incidences"], g1["n_colors"]) == (1089, 18178, 7)
    assert [e["n_stencils"] for e in g1["energies"]] == [3008, 2048, 2]
    assert (g2["n_vertices"], g2["n_incidences"]) == (4961, 96121)
    assert [e["n_stencils"] for e in g2["energies"]] == [121, 24000]
    assert (g3["n_vertices"], g3["n_incidences"], g3["n_colors"]) == (263169, 4717057, 7)
    assert [e["n_stencils"] for e in g3["energies"]] == [785408, 787456, 513]


@pytest.mark.skipif(O.ref_lib() is None, reason="reference checkout not present")
def test_literal_colouring_equals_compiled_reference():
    for obj in (scenes.cloth_cfg1(17), scenes.beam_cfg2(7, 4, 4), scenes.spring_cloth_cfg3(33),
                *scenes.patch_batch_cfg4(3, 8, 20, seed=9)):
        assert np.array_equal(O.color_vertices(obj), O.ref_color_vertices(obj))
        for e in obj.energies:
            k = [x is e for x in obj.energies].index(True)
            assert np.array_equal(O.Xpbd(obj, 1 / 60, 1, scenes.GRAVITY).stencil_colors(k), O.ref_color_stencils(e))


def test_vbd_full_ad_and_vertex_ad_trajectories_agree():
    obj = scenes.cloth_cfg1(9)
    a = O.Vbd(obj, 1 / 60, 1, 10, scenes.GRAVITY, O.FULL_AD)
    b = O.Vbd(obj, 1 / 60, 1, 10, scenes.GRAVITY, O.VERTEX_AD)
    for _ in range(3):
        a.step()
        b.step()
    assert np.abs(a.state()[0] - b.state()[0]).max() <= 1e-12
