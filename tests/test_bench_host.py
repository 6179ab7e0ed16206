"""bench.py's host-side logic, without a GPU: the roofline arithmetic, the
clock sampler's parsing and throttle-reason detection (a run that saw a
hardware or thermal slowdown is rejected), the committed traffic figure the
bench line quotes, the peak denominators and the contract's defaults."""
import json
import os
import sys

import pytest

import kvtest_util as U

sys.path.insert(0, U.ROOT)
import bench  # noqa: E402


def test_bytes_roofline_arithmetic():
    rec = {"ms": 2.0, "bytes": 3.0e9, "launches": 4}
    r = bench.bytes_roofline(rec, "k_mix", 6000.0, "measured")
    assert r["achieved"] == pytest.approx(1500.0)  # 3 GB in 2 ms = 1500 GB/s
    assert r["frac"] == pytest.approx(0.25)
    assert r["bytes_per_launch"] == pytest.approx(7.5e8)
    assert r["us_per_launch"] == pytest.approx(500.0)
    assert r["kernel"] == "k_mix" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert bench.bytes_roofline({"ms": 0.0, "bytes": 0.0, "launches": 0}, "k_mix", 6000.0, "measured") is None


def _clocks_from(rows):
    c = bench.Clocks(0)
    c.f.write("".join(rows))
    return c.summary()


def test_clock_summary_median_max_and_reasons():
    ok = "0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active\n"
    cap = "0, 1995, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n"
    s = _clocks_from([ok, ok, cap])
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    hot = "0, 1500, 2070, 700.0, 0x48, Not Active, Active, Not Active, Not Active\n"
    s = _clocks_from([ok, hot])
    assert s["reasons"] == ["hw_thermal_slowdown"]
    assert _clocks_from([])["reasons"] == ["unavailable"]


def test_traffic_figure_is_the_committed_capture():
    t = bench.traffic_per_launch(bench.DEFAULT_CONFIG)
    with open(os.path.join(U.ROOT, "profiles", f"k_gemm_tc_{bench.DEFAULT_CONFIG}.md")) as f:
        line = [ln for ln in f if ln.startswith("traffic_bytes_per_launch:")][0]
    assert t == float(line.split(":")[1]) and t > 0
    assert bench.traffic_per_launch("no-such-workload") is None


def test_peaks_come_from_the_measured_file():
    bf16, hbm, src = bench.peaks()
    p = os.path.join(U.ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        assert (bf16, hbm, src) == (float(d["bf16_tflops"]), float(d["hbm_gbs"]), "measured")
    else:
        assert src == "fallback"


def test_contract_defaults(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.config == bench.DEFAULT_CONFIG and a.impl == "ours"
