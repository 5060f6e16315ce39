"""The benchmark's derived figures point at committed evidence.

bench.py turns the ncu-measured DRAM traffic of one launch per LU kernel
(committed summaries under profiles/) into each kernel's `traffic`, and
names the kernel behind every profile category.  These checks run on the
CPU: every summary it cites exists, states its full ncu command with
--clock-control none, and its ratio is a plausible fraction of the
algorithmic bytes; every category maps to a kernel the library defines.
"""
import os
import re

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_traffic_ratios_cite_committed_ncu_summaries():
    assert bench.NCU_TRAFFIC_RATIO
    for cat, (ratio, source) in bench.NCU_TRAFFIC_RATIO.items():
        assert cat in bench.ROOF_KERNELS, cat
        path = os.path.join(ROOT, source)
        assert os.path.isfile(path), source
        text = open(path).read()
        assert "ncu " in text and "--clock-control none" in text, source
        assert bench.ROOF_KERNELS[cat][0].split("<")[0] in text, (cat, source)
        assert 0.3 < ratio < 1.5, (cat, ratio)


def test_roofline_kernels_exist_in_the_sources():
    src = ""
    csrc = os.path.join(ROOT, "kadath_frontera_gb300", "csrc")
    for name in os.listdir(csrc):
        if name.endswith((".cu", ".cpp", ".hpp")):
            src += open(os.path.join(csrc, name)).read()
    for cat, (kernel, what) in bench.ROOF_KERNELS.items():
        base = kernel.split("<")[0]
        assert re.search(r"\b" + re.escape(base) + r"\b", src), (cat, kernel)
        assert what


def test_roofline_arithmetic():
    st = {"launches": 100, "ms": 10.0, "work": 100 * 5.0e6}
    out = bench.roofline_for("lu_swap_trsm", st, {"hbm_gbs": 6000.0}, "measured", 1.0)
    assert abs(out["avg_launch_ms"] - 0.1) < 1e-12
    assert abs(out["achieved"] - 5.0e6 / 1e-4 / 1e9) < 1e-9  # GB/s
    assert abs(out["frac"] - out["achieved"] / 6000.0) < 1e-12
    ratio = bench.NCU_TRAFFIC_RATIO["lu_swap_trsm"][0]
    assert abs(out["traffic"] - ratio * 5.0e6) < 1e-6
