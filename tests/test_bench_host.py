"""Host-side pieces of bench.py (no GPU): the clock and throttle summary of
the nvidia-smi samples taken during the timed region."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


def _rows(lines):
    return [[x.strip() for x in ln.split(",")] for ln in lines]


def test_clock_summary_median_and_reasons():
    c = bench.Clocks(0)
    c.rows = _rows([
        "0, 2070, 2070, 1100.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2032, 2070, 1398.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2055, 2070, 1250.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
    ])
    s = c.summary()
    assert s["sm_mhz"] == 2055 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_reports_thermal_and_unsampled():
    c = bench.Clocks(0)
    assert c.summary()["reasons"] == ["unsampled"]
    c.rows = _rows(["0, 1500, 2070, 900.0, 0x20, Not Active, Active, Not Active, Not Active",
                    "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]"])
    s = c.summary()
    assert s["sm_mhz"] == 1500 and s["reasons"] == ["hw_thermal_slowdown"] and s["samples"] == 2
