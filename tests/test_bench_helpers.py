"""bench.py's host-side pieces on the CPU: the algorithmic bytes of the 513x513 spring cloth
(one compulsory pass per iteration, 243 B per vertex-solve; one XPBD substep), the DRAM
traffic per sweep recorded from the committed ncu summaries of the VBD kernels, and the
summary of the clocks sampled during the timed region."""
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


def test_xpbd_algorithmic_bytes_of_the_513_cloth():
    """One substep's compulsory bytes: 787,456 spring records x 20 B, 785,408 bending records
    x 32 B, 513 anchor records x 28 B, and 132 B of vertex state per vertex."""
    bench = pytest.importorskip("bench")
    from spg_gb300 import scenes as S
    obj = S.spring_cloth(513).objects[0]
    expect = 20 * 787456 + 32 * 785408 + 28 * 513 + 132 * 263169
    assert bench.xpbd_algorithmic_bytes_per_substep(obj) == expect == 75634848


def test_clock_sampler_summary():
    """The clocks record of the timed region: median SM clock, the highest max clock, and the
    throttle reasons seen active in any sample; malformed and N/A lines are skipped."""
    bench = pytest.importorskip("bench")
    c = bench.ClockSampler(0)
    c.lines = [
        "2070, 2070, 910.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "1980, 2070, 1390.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "2055, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "[N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]",
        "garbage",
    ]
    got = c.stop()
    assert got == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    empty = bench.ClockSampler(0)
    assert empty.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_cpu_baseline_runs_whole_sweeps_of_the_oracle():
    """The cpu_baseline leg: at least one whole colour sweep of the 513x513 cloth on every host
    thread, reported as vertex-solves/s of the oracle ("port")."""
    bench = pytest.importorskip("bench")
    b = bench.cpu_baseline(0.1)
    assert b["kind"] == "port" and b["unit"] == bench.UNIT and b["cores"] == (os.cpu_count() or 1)
    assert b["value"] > 0 and "263169 vertex-solves" in b["sample"]
