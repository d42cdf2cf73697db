"""bench.py's measurement arithmetic on the CPU: the algorithmic bytes its
roofline divides by (from the library's host-only planner), the radix-4
flop count, the clock record that decides whether a run is rejected, and
the peak it reports against."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import cvmatch_gb300 as cvm  # noqa: E402


def test_fft_flops_counts_the_radix4_engine():
    assert bench.fft_flops(4) == 34                   # one radix-4 butterfly
    assert bench.fft_flops(8) == 4 * 4 + 34 * 2       # radix-2 head, then one radix-4 stage
    assert bench.fft_flops(1024) == 34 * 256 * 5      # five radix-4 stages
    assert bench.fft_flops(2048) == 4 * 1024 + 34 * 512 * 5


def test_match_models_pin_the_1920x1080_colour_match():
    import ctypes as C
    L = cvm.lib()
    out = (C.c_int32 * 6)()
    assert L.cvm_plan(96, 32, 1920 - 96 + 1, 1080 - 32 + 1, out) == 0
    assert (out[0], out[1], out[5]) == (1024, 256, 10)  # dftW, dftH, tiles
    fast, exact = bench.match_models(L, "fast"), bench.match_models(L, "exact")
    frame = 1920 * 1080 * 4
    hp = -(-(1920 - 96 + 1) // 32) * 32
    assert fast["k_prep"][0] == frame
    assert fast["k_hsum"][0] == frame + 1080 * hp * 16
    # the per-kernel algorithmic bytes behind the bench line's roofline
    assert fast["k_fwd_rows"][0] == 39351536
    assert fast["k_cols_fwd_sum_inv"][0] == 69817248
    assert fast["k_inv_rows"][0] == 16308932
    assert fast["k_vstats"][0] == 100163300
    # the exact form's inverse rows read every channel and a (t, den) lane
    rw, rh = 1920 - 96 + 1, 1080 - 32 + 1
    assert exact["k_inv_rows"][0] - rw * rh * 8 == 3 * (fast["k_inv_rows"][0] - rw * rh * 4)
    assert exact["k_vstats"][0] - fast["k_vstats"][0] == rw * rh * 4


def test_measured_traffic_covers_the_roofline_kernel():
    for form, kernel in (("fast", "k_cols_fwd_sum_inv"), ("exact", "k_cols_fwd_mul_inv")):
        t = bench.measured_traffic(form)
        assert t.get(kernel, 0) > 0
        assert all(v > 0 for v in t.values())


def test_clock_record_flags_throttling():
    s = bench.ClockSampler(0)
    s.lines = ["2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
               "2055, 2070, 1390.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "2070, 2070, 1395.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "garbage line",
               "[N/A], 2070, 10, 0x0, Not Active, Not Active, Not Active, Not Active"]
    r = s.summary()
    assert r["samples"] == 3 and r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]
    s.lines.append("1500, 2070, 700, 0x40, Not Active, Active, Not Active, Not Active")
    assert "hw_thermal_slowdown" in s.summary()["reasons"]


def test_clock_record_splits_the_timed_region():
    s = bench.ClockSampler(0)
    s.lines = [(1.0, "2070, 2070, 900, 0x0, Not Active, Not Active, Not Active, Not Active"),
               (2.0, "2055, 2070, 1300, 0x0, Not Active, Not Active, Not Active, Not Active"),
               (2.5, "2040, 2070, 1300, 0x0, Not Active, Not Active, Not Active, Not Active"),
               (3.0, "2025, 2070, 1300, 0x0, Not Active, Not Active, Not Active, Not Active"),
               (9.0, "2070, 2070, 500, 0x0, Not Active, Not Active, Not Active, Not Active")]
    r = s.summary(1.5, 3.2)
    assert r["samples"] == 5 and r["samples_timed"] == 3 and r["sm_mhz_timed"] == 2040.0
    assert bench.ClockSampler(0).period_ms <= 25  # several samples inside a C4 run's ~0.2 s of timed steps


def test_peak_is_measured_or_the_stated_fallback():
    peak, kind = bench.measured_peaks()
    assert kind in ("measured", "fallback") and peak > 0
    if kind == "fallback":
        assert peak == 6800.0
