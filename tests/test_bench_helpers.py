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


def test_frame_bytes_of_the_plain_small_frame():
    """The frame-level algorithmic bytes of the plain small frame: vertex array (2,145 x 64 B),
    indices (3,968 triangles), the 256^2 checker's mip chain and 1024x768 colour + depth written
    once: about 6.8 MB."""
    from softglrender_gb300 import scenes as S
    sc = S.config_plain_small()
    d = sc.passes[0].draws[0]
    tex = sum(max(1, 256 >> l) ** 2 * 4 for l in range(9))
    want = d.vertexes.nbytes + 4 * len(d.indices) + tex + 1024 * 768 * 8
    assert bench.frame_bytes(sc) == want
    assert 6.6e6 < want < 7.0e6


def test_raster_launch_bytes_counts_reads_only_when_not_cleared():
    from softglrender_gb300 import api as A
    opaque = A.RenderStates(depthTest=True, depthMask=True)
    blend = A.RenderStates(blend=True, depthTest=True, depthMask=False)
    n = 64 * 32 * 4
    a = bench.raster_launch_bytes(64, 32, 4, True, opaque, 0, 0, 8)
    assert a == n * 4 + 64 * 32 * 4 + n * 4                       # colour + resolved + depth write
    b = bench.raster_launch_bytes(64, 32, 4, False, blend, 10, 5, 8)
    assert b == n * 4 + 64 * 32 * 4 + n * 4 + n * 4 + 10 * 132 + 5 * 3 * 8 * 4   # + colour, depth reads


def test_issue_roofline_from_the_committed_profile():
    w = bench.profiled_value("k_raster_cov_pbr_ibl_1080p_msaa4.md", "warp_instructions_per_launch")
    assert isinstance(w, int) and w > 1_000_000
    r = bench.issue_roofline(w, 0.2, 2000.0)
    assert r["peak_warp_inst_per_s"] == 152 * 4 * 2000e6
    assert abs(r["frac"] - w / 0.2e-3 / (152 * 4 * 2000e6)) < 1e-3
    assert bench.issue_roofline(None, 0.2, 2000.0) is None
