"""Host-side helpers of bench.py, on CPU: the clock record that decides whether a
timed run is kept (throttle reasons, median SM clock) and the bounded CPU
sample of the oracle baseline (stride refinement, middle pair of each stride)."""
import os
import tempfile

import pytest

import bench


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _sampler_with(lines):
    s = bench.ClockSampler(0)
    fd, s.path = tempfile.mkstemp(suffix=".csv")
    s.fh = os.fdopen(fd, "w")
    s.fh.write("\n".join(lines) + "\n")
    s.proc = _FakeProc()
    return s


def test_clock_record_median_and_reasons():
    # nvidia-smi --format=csv,noheader,nounits: index, sm, max sm, power, active mask, 4 reasons
    lines = [
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1300.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1350.2, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 10.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = _sampler_with(lines)
    rec = s.stop()
    assert not os.path.exists(s.path)
    assert rec == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_clock_record_flags_thermal_slowdown():
    lines = ["0, 1500, 2070, 1390.0, 0x48, Active, Not Active, Active, Not Active"] * 4
    rec = _sampler_with(lines).stop()
    assert rec["sm_mhz"] == 1500.0
    assert rec["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_clock_record_without_samples_is_none():
    assert _sampler_with(["not,a,sample"]).stop() is None
    assert bench.ClockSampler(0).stop() is None   # never started


@pytest.mark.parametrize("full_s,budget_s", [(400.0, 20.0), (30.0, 20.0), (5.0, 20.0), (2000.0, 10.0)])
def test_bounded_sample_fills_half_the_budget(full_s, budget_s):
    calls = []

    def run(stride, offset):
        calls.append((stride, offset))
        return full_s / stride, {"stride": stride}

    est, stride, info = bench.sampled(run, budget_s)
    # every timed sample takes the middle pair of its stride
    assert all(off == st // 2 for st, off in calls)
    assert info["stride"] == stride and calls[-1][0] == stride
    # the estimate scales the sample back to the whole loop
    assert est == pytest.approx(full_s)
    # the sample fills at least half the budget, or is the whole loop
    assert stride == 1 or full_s / stride >= 0.5 * budget_s
    assert len(calls) <= 6
