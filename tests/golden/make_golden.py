"""Generates tests/golden/coloring_golden.json from the reference's own greedy colouring
(spg/source/utils/graphColoring.cpp compiled into oracle/_ref by oracle/build.py) on the
benchmark scenes built by the oracle's restatement of the reference's scene builders.

Run where the reference checkout is present: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as ob  # noqa: E402
from oracle import pyoracle as O  # noqa: E402
from tests import scenes  # noqa: E402


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def entry(obj, full: bool) -> dict:
    colors = O.ref_color_vertices(obj)
    d = {"n_vertices": int(obj.nv), "n_colors": int(colors.max()) + 1,
         "histogram": np.bincount(colors).tolist(), "sha256": digest(colors),
         "energies": [{"type": int(e.type), "n_stencils": int(e.n)} for e in obj.energies],
         "n_incidences": int(sum(e.stencils.size for e in obj.energies)),
         "stencil_colors": [{"n_colors": int(c.max()) + 1 if c.size else 0, "sha256": digest(c)}
                            for c in (O.ref_color_stencils(e) for e in obj.energies)]}
    if full:
        d["colors"] = colors.tolist()
    return d


def main():
    ob.build()
    if O.ref_lib() is None:
        raise SystemExit("the reference checkout is needed to compile its colouring")
    out = {"generator": "tests/golden/make_golden.py",
           "source": "reference spg/source/utils/graphColoring.cpp (colorVertices, colorStencils)",
           "scenes": {}}
    out["scenes"]["cloth_33"] = entry(scenes.cloth_cfg1(33), True)
    out["scenes"]["beam_41x11x11_6tet"] = entry(scenes.beam_cfg2(), False)
    out["scenes"]["beam_9x4x4_5tet"] = entry(O.build_tet_beam(62.5, 0.2, 0.075, 0.075, 9, 4, 4, 1e6, 0.45, 1e4, 5),
                                              True)
    out["scenes"]["spring_cloth_65"] = entry(scenes.spring_cloth_cfg3(65), True)
    out["scenes"]["spring_cloth_513"] = entry(scenes.spring_cloth_cfg3(513), False)
    out["scenes"]["patch_batch_8"] = [entry(o, False) for o in scenes.patch_batch_cfg4(8, 16, 128, seed=2024)]
    with open(os.path.join(HERE, "coloring_golden.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "coloring_golden.json"))


if __name__ == "__main__":
    main()
