"""bench.py's clock record: nvidia-smi samples are kept only inside the timed
region's wall-clock window (the one nearest its middle when the region is
shorter than the sampling interval), and throttle reasons seen inside it are
reported.  Parsed from a written sample file; no GPU or nvidia-smi needed."""
import datetime
import os
import sys
import time

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _line(t, sm, power_cap=False):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    cap = "Active" if power_cap else "Not Active"
    return f"{ts}, 0, {sm}, 2070, 900.00, 0x0, Not Active, Not Active, Not Active, {cap}\n"


def test_samples_inside_the_window_only(tmp_path):
    sys.path.insert(0, REPO)
    import bench

    c = bench.ClockSampler(0)
    c.path = str(tmp_path / "clocks.csv")
    t0 = time.time()
    with open(c.path, "w") as f:
        f.write("garbage line\n")
        for k in range(10):  # one sample every 20 ms; 1,800 MHz and power cap outside the window
            inside = 3 <= k <= 6
            f.write(_line(t0 + 0.02 * k, 2070 if inside else 1800, power_cap=k == 8))
    c.mark(t0 + 0.05, t0 + 0.13)
    r = c.summary()
    assert r["samples"] == 4 and r["sm_mhz"] == 2070.0 and r["reasons"] == [], r
    # a window shorter than the interval: the sample nearest its middle
    c.mark(t0 + 0.161, t0 + 0.165)
    r = c.summary()
    assert r["samples"] == 1 and r["reasons"] == ["sw_power_cap"] and r["sm_mhz"] == 1800.0, r
