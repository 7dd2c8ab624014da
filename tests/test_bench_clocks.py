"""bench.py's clock record: the summary of the nvidia-smi samples taken over the warm-up and
the timed region (median SM clock, the largest maximum clock, the number of samples, every
throttle reason seen active), read from a sample file written here -- no GPU and no
nvidia-smi needed."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Proc:
    """Stands in for the sampler's nvidia-smi process."""


def _sampler(tmp_path, lines):
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "clocks.csv")
    with open(s.path, "w") as f:
        f.write("\n".join(lines) + "\n")
    s.proc = _Proc()
    return s


def test_summary_of_samples(tmp_path):
    # index, sm, max sm, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, 2055, 2070, 1380.0, 0x4, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, [N/A], 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
             "garbage line"]
    out = _sampler(tmp_path, lines).summary()
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2070.0
    assert out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_slowdown_reasons_are_reported(tmp_path):
    lines = ["0, 1500, 2070, 1400.0, 0x8, Active, Not Active, Active, Not Active",
             "0, 1600, 2070, 1400.0, 0x8, Not Active, Active, Not Active, Not Active"]
    out = _sampler(tmp_path, lines).summary()
    assert out["samples"] == 2
    assert out["sm_mhz"] == 1550.0
    assert out["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_no_samples_and_no_sampler(tmp_path):
    assert _sampler(tmp_path, ["not a sample"]).summary()["reasons"] == ["no samples"]
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "absent.csv")
    assert s.summary()["reasons"] == ["nvidia-smi unavailable"]
