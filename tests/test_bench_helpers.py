"""bench.py's roofline inputs on the CPU: the algorithmic bytes of the 513x513 spring cloth
(one compulsory pass per iteration, 243 B per vertex-solve) and the DRAM traffic per sweep
recorded from the committed ncu summaries of the VBD kernels."""
import json
import os

import pytest

from tests import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_algorithmic_bytes_of_the_513_cloth():
    bench = pytest.importorskip("bench")
    obj = scenes.spring_cloth_cfg3(513)
    # 263,169 vertices x 48 B, 263,170 offsets x 4 B, 4,717,057 incidences x 4 B, and the
    # records: 787,456 springs x 16 B, 785,408 bending stencils x 24 B, 513 anchors x 20 B.
    expect = 48 * 263169 + 4 * 263170 + 4 * 4717057 + 16 * 787456 + 24 * 785408 + 20 * 513
    assert bench.algorithmic_bytes_per_iteration(obj) == expect == 64012368
    assert abs(expect / 263169 - 243.24) < 0.01


@pytest.mark.parametrize("kernel", ["vbd_flow_kernel", "vbd_tile_kernel", "vbd_color_kernel"])
def test_recorded_traffic_is_near_the_algorithmic_bytes(kernel):
    """Each summary's DRAM bytes per sweep are what bench.py reports as roofline.traffic; a
    value far above the compulsory 64.0 MB would mean re-reads, far below a wrong capture."""
    bench = pytest.importorskip("bench")
    with open(os.path.join(ROOT, "profiles", f"{kernel}_spring_cloth_513.json")) as f:
        rec = json.load(f)
    assert "--clock-control none" in rec["command"]
    t = bench._traffic_per_iteration(kernel)
    assert t == float(rec["dram_bytes_per_sweep"])
    assert 0.9 * 64012368 < t < 40 * 64012368
