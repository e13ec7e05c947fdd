"""Host-side pieces of bench.py that need no GPU: the step-count defaults
of the two arms and the reading of the clock samples (throttle reasons,
loaded-sample median)."""

import sys

import pytest


@pytest.fixture(scope="module")
def bench():
    import bench as b

    return b


def test_step_defaults(bench, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    assert bench.parse_args().steps == 50
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    assert bench.parse_args().steps == 5
    monkeypatch.setattr(sys, "argv", ["bench.py", "--steps", "7", "--impl", "reference"])
    assert bench.parse_args().steps == 7


def row(sm, power, hw="Not Active", hwt="Not Active", swt="Not Active", pcap="Not Active", smax=2070):
    return f"0, {sm}, {smax}, {power}, 0x0, {hw}, {hwt}, {swt}, {pcap}"


def test_clock_summary_loaded_median_and_reasons(bench):
    lines = [row(420, 150.0), row(2070, 400.0), row(2070, 410.0), row(1980, 405.0, pcap="Active"),
             "garbage", row(600, 160.0)]
    c = bench.Clocks.summarize(lines)
    assert c["samples"] == 5
    assert c["sm_mhz"] == 2070.0  # median of the loaded samples (power >= half the peak)
    assert c["sm_max_mhz"] == 2070.0
    assert c["power_w_max"] == 410.0
    assert c["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_slowdowns(bench):
    c = bench.Clocks.summarize([row(2070, 400.0), row(1500, 390.0, hw="Active", hwt="Active", swt="Active")])
    assert c["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert bench.Clocks.summarize([]) is None
