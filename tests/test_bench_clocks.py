"""bench.py's clock record keeps only the nvidia-smi samples whose
timestamps fall inside the timed region, and reports throttle reasons seen
there (no GPU: the sampler's rows are set directly)."""
import datetime
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def row(t, mhz, power_cap=False, thermal=False):
    ts = t.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    na, act = "Not Active", "Active"
    return [ts, "0", str(mhz), "2070", "900.00", "0x0", na, na, act if thermal else na, act if power_cap else na]


def test_samples_outside_the_timed_region_are_dropped():
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    s = bench.ClockSampler(0)
    s.rows = [row(t0 - datetime.timedelta(seconds=0.2), 300, thermal=True),  # idle, before
              row(t0 + datetime.timedelta(seconds=0.1), 2070),
              row(t0 + datetime.timedelta(seconds=0.3), 2055, power_cap=True),
              row(t0 + datetime.timedelta(seconds=0.5), 2070),
              row(t0 + datetime.timedelta(seconds=1.2), 345, thermal=True)]  # after
    s.t0, s.t1 = t0, t0 + datetime.timedelta(seconds=1.0)
    c = s.summary()
    assert c["samples"] == 3 and c["samples_total"] == 5
    assert c["sm_mhz"] == 2070.0 and c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == ["sw_power_cap"]


def test_no_sample_inside_is_reported_as_unsampled():
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    s = bench.ClockSampler(0)
    s.rows = [row(t0 - datetime.timedelta(seconds=1), 2070), ["garbage"]]
    s.t0, s.t1 = t0, t0 + datetime.timedelta(seconds=0.01)
    c = s.summary()
    assert c["samples"] == 0 and c["reasons"] == ["unsampled"] and c["sm_mhz"] is None
