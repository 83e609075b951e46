"""The bench's clock record: only nvidia-smi readings stamped inside the timed
region count, throttle reasons are collected from them, and a region shorter
than the sampling period takes the reading nearest to it (CPU only, fake
readings)."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402

IDLE = "0, 1000, 2070, 100, 0x0, Not Active, Not Active, Not Active, Not Active"
CAP = "0, 2070, 2070, 900, 0x4, Not Active, Not Active, Not Active, Active"
LOAD = "0, 2060, 2070, 900, 0x0, Not Active, Not Active, Not Active, Not Active"
SLOW = "0, 500, 2070, 100, 0x8, Active, Not Active, Not Active, Not Active"


def _sampler(lines, t0, t1):
    c = bench.ClockSampler(0)
    c.lines = list(lines)
    c.t0, c.t1 = t0, t1
    return c


def test_only_readings_inside_the_region_count():
    c = _sampler([(9.0, IDLE), (10.05, CAP), (10.15, LOAD), (15.0, SLOW)], 10.0, 10.2)
    s = c.summary()
    assert s["samples"] == 2
    assert s["sm_mhz"] == 2065.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]  # the hw_slowdown reading came after the region
    assert s["region_s"] == 0.2


def test_short_region_takes_the_nearest_reading():
    c = _sampler([(9.0, IDLE), (10.05, LOAD), (15.0, SLOW)], 14.9, 14.91)
    s = c.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 500.0 and s["reasons"] == ["hw_slowdown"]


def test_no_readings_is_reported_unsampled():
    s = _sampler([], None, None).summary()
    assert s["samples"] == 0 and s["reasons"] == ["unsampled"] and s["sm_mhz"] is None


def test_malformed_lines_are_skipped():
    c = _sampler([(10.05, "garbage"), (10.1, "0, [N/A], 2070, 1, 0x0, a, b, c, d"), (10.15, LOAD)], 10.0, 10.2)
    s = c.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 2060.0 and s["reasons"] == []
