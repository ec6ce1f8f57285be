"""Host-side pieces of bench.py's report, without a GPU: the clock record
taken during the timed region and the algorithmic byte and flop counts
behind the roofline lines."""
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def row(sm, sm_max=2070, hw="Not Active", hw_th="Not Active", sw_th="Not Active", pcap="Not Active"):
    return f"0, {sm}, {sm_max}, 812.40, 0x0000000000000000, {hw}, {hw_th}, {sw_th}, {pcap}\n"


def test_clock_record_median_max_and_reasons():
    lines = [row(2070), row(1965, pcap="Active"), row(2070), "garbage line\n", row(2055)]
    out = bench.ClockSampler.summarize(lines)
    assert out["samples"] == 4
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_record_reports_every_slowdown_reason():
    lines = [row(1410, hw="Active"), row(1410, hw_th="Active", sw_th="Active")]
    out = bench.ClockSampler.summarize(lines)
    assert out["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert out["sm_mhz"] == 1410.0


def test_clock_record_without_samples_is_none():
    assert bench.ClockSampler.summarize([]) is None
    assert bench.ClockSampler.summarize(["[N/A], [N/A]\n"]) is None


def test_algorithmic_schur_bytes_counts_each_stream_once():
    # one observation, one point, one camera with p_c = 12, n = 12, FP32
    no, np_, n, p_c, s = 1, 1, 12, 12, 4
    reads = no * (16 + 12) + np_ * (24 + 48 + 4) + 1 * p_c * 8 + no * 6 * p_c * s
    writes = no * (9 * p_c + 8) * s + np_ * 9 * s + (n * n // 2) * s + n * s
    assert bench.algorithmic_schur_bytes(no, np_, n, p_c, s) == reads + writes
    # linear in the observations at a fixed camera system
    a = bench.algorithmic_schur_bytes(1000, 100, 600, 12, 4)
    b = bench.algorithmic_schur_bytes(2000, 100, 600, 12, 4)
    assert b - a == 1000 * (16 + 12 + 6 * 12 * 4 + (9 * 12 + 8) * 4)


def test_factor_flops():
    assert bench.factor_flops(3) == 27 / 3 + 18
    assert abs(bench.factor_flops(5988) - 7.1640575712e10) < 1e3
