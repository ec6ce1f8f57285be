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


def test_algorithmic_schur_bytes_follow_the_survey_formula():
    # N_o (2s + 4 + 3 p_c s) + N_p (3s + 6s) + nnzb(S) p_c^2 s
    no, np_, nnzb, p_c, s = 1_999_428, 200_000, 125_250, 12, 4
    expect = no * (2 * s + 4 + 3 * p_c * s) + np_ * 9 * s + nnzb * p_c * p_c * s
    assert bench.algorithmic_schur_bytes(no, np_, nnzb, p_c, s) == expect
    assert abs(expect - 0.3912e9) < 0.001e9  # the medium workload's 0.391 GB
    a = bench.algorithmic_schur_bytes(1000, 100, 600, 12, 4)
    b = bench.algorithmic_schur_bytes(2000, 100, 600, 12, 4)
    assert b - a == 1000 * (8 + 4 + 3 * 12 * 4)


def test_covisible_blocks_counts_camera_pairs_once():
    # point 0 seen by cameras 0, 2, 3; point 1 by 2, 3; point 2 by 1
    pt = [0, 0, 0, 1, 1, 2]
    cam = [0, 2, 3, 2, 3, 1]
    # diagonal (0,0) (1,1) (2,2) (3,3) + (2,0) (3,0) (3,2)
    assert bench.covisible_blocks(pt, cam, 4) == 7
    # order of the observations does not matter
    perm = [5, 3, 0, 4, 1, 2]
    assert bench.covisible_blocks([pt[i] for i in perm], [cam[i] for i in perm], 4) == 7


def test_factor_flops():
    assert bench.factor_flops(3) == 27 / 3 + 18
    assert abs(bench.factor_flops(5988) - 7.1640575712e10) < 1e3
