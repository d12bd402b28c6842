"""Host logic of bench.py: the clock record keeps only the nvidia-smi samples
stamped inside the timed region (plus the first after it) and reports the
throttle reasons seen there."""
import datetime
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    # imported inside the tests: bench.py sets CUDA environment defaults at
    # import, which must not leak into the collection of the GPU tests
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def _write(path, t0, mhz, power_cap_at=()):
    lines = []
    for i, f in enumerate(mhz):
        t = t0 + datetime.timedelta(milliseconds=50 * i)
        cap = "Active" if i in power_cap_at else "Not Active"
        lines.append(f"{t.strftime('%Y/%m/%d %H:%M:%S.%f')[:-3]}, 0, {f}, 2070, 900.0, 0x0, Not Active, "
                     f"Not Active, Not Active, {cap}")
    lines.append("garbage line")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def _sampler(path):
    c = _bench().ClockSampler(0)
    c.path = str(path)
    c.proc = object()   # as if nvidia-smi had run
    return c


def test_clock_summary_keeps_the_timed_region(tmp_path):
    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5)
    _write(tmp_path / "c.csv", t0, [1000, 1100, 2070, 2070, 2060, 2070, 1200, 1300], power_cap_at=(0, 7))
    c = _sampler(tmp_path / "c.csv")
    # region covers samples 2..4; sample 5 is the first after it
    c.region(t0 + datetime.timedelta(milliseconds=90), t0 + datetime.timedelta(milliseconds=210))
    s = c.summary()
    assert s["samples"] == 4
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == []          # the power-cap samples lie outside the region
    c.window = None
    s = c.summary()
    assert s["samples"] == 8 and s["reasons"] == ["sw_power_cap"]


def test_clock_summary_without_nvidia_smi(tmp_path):
    c = _bench().ClockSampler(0)
    c.path = str(tmp_path / "missing.csv")
    s = c.summary()
    assert s["sm_mhz"] is None and s["reasons"] == ["nvidia-smi unavailable"]


def test_clock_summary_unparsed_timestamps_keep_every_sample(tmp_path):
    path = tmp_path / "c.csv"
    path.write_text("Fri Dec 4 06:22:03 2026, 0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, "
                    "Not Active\n" * 3)
    c = _sampler(path)
    t0 = datetime.datetime(2026, 1, 2)
    c.region(t0, t0 + datetime.timedelta(seconds=1))
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0
