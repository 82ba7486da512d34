"""Host-side logic of the benchmark and the served stream, without a GPU.

The clock record decides whether a bench line is valid: a run that saw
hw_slowdown, hw_thermal_slowdown or sw_thermal_slowdown inside the timed
window must report it, and samples outside the window must not count.  The
force pass's roofline figures come from the committed ncu captures.  The
served bench compares itself with the plain path through a first-come
first-served latency model fitted to measured run times.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from tecs_gb300 import served  # noqa: E402
from tecs_gb300 import workloads as wl  # noqa: E402


def clock_line(mhz, reasons=()):
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    flags = ["Active" if nm in reasons else "Not Active" for nm in names]
    return f"0, {mhz}, 2070, 900.00, 0x0000000000000000, " + ", ".join(flags) + "\n"


def test_clock_summary_counts_only_the_timed_window(tmp_path):
    p = tmp_path / "clocks.csv"
    lines = [clock_line(1200, ("hw_slowdown",))]  # before the timed region
    lines += [clock_line(2070), clock_line(2055, ("sw_power_cap",)), clock_line(2070)]
    lines += [clock_line(900, ("hw_thermal_slowdown",))]  # after it
    p.write_text("".join(lines))
    c = bench.Clocks(0)
    c.path = str(p)
    c.lo, c.hi = 1, 4
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 3
    # the record is read once: a second call returns the same summary
    assert c.summary() == s


def test_clock_summary_reports_throttling_inside_the_window(tmp_path):
    p = tmp_path / "clocks.csv"
    p.write_text(clock_line(1800, ("hw_thermal_slowdown", "sw_thermal_slowdown")) + clock_line(2070))
    c = bench.Clocks(0)
    c.path = str(p)
    c.lo, c.hi = 0, 2
    s = c.summary()
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == pytest.approx(1935.0)


def test_clock_summary_without_samples():
    c = bench.Clocks(0)
    assert c.summary()["reasons"] == ["unsampled"]


def test_pass_figures_come_from_the_committed_captures():
    assert bench.pass_profile("spheroid", "pass_dram_bytes_per_cell") == pytest.approx(21.78)
    assert bench.pass_profile("spheroid", "pass_warp_inst_per_cell") == pytest.approx(140.96)
    assert bench.pass_profile("sheet", "pass_warp_inst_per_cell") == pytest.approx(289.0)
    assert bench.pass_profile("small", "pass_warp_inst_per_cell") is None
    assert bench.traffic_per_pass("sheet") == pytest.approx(71.6)


def test_fcfs_latency_model_fits_and_queues():
    # run time = steps * (a + b * cells) + c, sampled exactly
    a, b, c = 2e-5, 4e-10, 3e-3
    rows = [(n, k, k * (a + b * n) + c) for n, k in ((1000, 100), (50_000, 400), (200_000, 900), (800_000, 250))]
    reqs = [wl.Request(arrival_s=0.0, n=100_000, steps=500, model="spring", integrator="heun", seed=0),
            wl.Request(arrival_s=0.01, n=10_000, steps=100, model="spring", integrator="euler", seed=1),
            wl.Request(arrival_s=5.0, n=10_000, steps=100, model="polarity", integrator="heun", seed=2)]
    m = served.plain_fcfs_latency(reqs, rows)
    np.testing.assert_allclose(m["model_s_per_step"], [a, b, c], rtol=1e-6)
    t0 = 500 * (a + b * 100_000) + c
    t1 = 100 * (a + b * 10_000) + c
    # the second request waits for the first; the third arrives to an idle server
    lat = np.array([t0, t0 + t1 - 0.01, t1])
    assert m["p50_s"] == pytest.approx(float(np.percentile(lat, 50)))
    assert m["makespan_s"] == pytest.approx(5.0 + t1)
