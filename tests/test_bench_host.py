"""Host logic of bench.py that needs no GPU: the clock record taken during
the timed region (median SM clock, and every throttle reason seen Active,
which marks a run taken under hardware or thermal slowdown)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_clock_summary_reads_throttle_reasons():
    sys.path.insert(0, ROOT)
    import bench
    lines = ["0, 2070, 2070, 800.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "0, 1980, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 900.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "garbage line", "0, [N/A], 2070, 1.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c = bench.ClockSampler.summarize(lines)
    assert c["sm_mhz"] == 2070.0 and c["sm_max_mhz"] == 2070.0 and c["samples"] == 3
    assert c["reasons"] == ["sw_power_cap"]
    hot = ["0, 1500, 2070, 1400.0, 0x0000000000000048, Active, Not Active, Active, Not Active"]
    assert bench.ClockSampler.summarize(hot)["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_lapack_context_figure_lists_both_libraries():
    sys.path.insert(0, ROOT)
    import bench
    c = bench.cpu_lapack(8192, 32)
    assert c["value"] > 0 and c["unit"] == "TFLOP/s" and c["cores"] >= 1
    assert len(c["candidates"]) == 2 and c["kind"] in c["candidates"]
    assert c["seconds"] == min(v for v in c["candidates"].values() if isinstance(v, float))
