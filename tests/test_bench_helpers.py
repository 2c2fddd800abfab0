"""Host-side helpers of bench.py that run without a GPU: the ncu traffic figure of the roofline
kernel read from its committed summary, and the clock-sample summary."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_roofline_traffic_comes_from_the_committed_profile():
    t = bench.profiled_traffic()
    assert isinstance(t, int) and 1_000_000 < t < 1_000_000_000
    with open(os.path.join(ROOT, "profiles", "k_raster_cov_pbr_ibl_1080p_msaa4.md")) as f:
        text = f.read()
    # the per-launch figure equals the read + write rows of the same capture
    rows = {}
    for line in text.splitlines():
        for key in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            if line.startswith(f"| {key} |"):
                rows[key] = float(line.split("|")[2].split()[0])
    assert set(rows) == {"dram__bytes_read.sum", "dram__bytes_write.sum"}
    assert abs(sum(rows.values()) * 1e6 - t) < 0.01e6


def test_missing_profile_gives_no_traffic():
    assert bench.profiled_traffic("no_such_profile.md") is None


def test_clock_summary_reports_median_under_load_and_reasons():
    cs = bench.ClockSampler(0)
    cs.lines = [
        "1000, 2070, 300.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "2070, 2070, 950.0, 0x4, Not Active, Not Active, Not Active, Active",
        "2055, 2070, 940.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    s = cs.summary()
    assert s["samples"] == 4
    assert s["sm_max_mhz"] == 2070.0
    assert s["sm_mhz"] == 2070.0            # the lowest quarter (idle samples) is left out
    assert s["reasons"] == ["sw_power_cap"]
    assert bench.ClockSampler(0).summary()["samples"] == 0
