"""Host-side logic of bench.py that needs no GPU: the ncu traffic figures
read from the committed profile summaries (scaled to the benched workload by
algorithmic bytes), the clock record of the timed region, and the bounded
timing windows."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_profile_traffic_of_each_profiled_workload():
    # a profile read at its own algorithmic bytes gives its captured traffic
    t, src = bench.profile_traffic("c2", "MIXED", 140024280)
    assert src == "profiles/k_step_mixed_c2.md"
    assert t == pytest.approx(165195520, rel=1e-9)
    t, src = bench.profile_traffic("c2", "FP64", 246151608)
    assert src == "profiles/k_step_fp64_c2.md" and t == pytest.approx(257220864, rel=1e-9)
    # the C4 capture ran 64 of the 256 plates: scaled by the algorithmic bytes
    t64, _ = bench.profile_traffic("c4", "MIXED", 323720384)
    t256, src = bench.profile_traffic("c4", "MIXED", 4 * 323720384)
    assert src == "profiles/k_step_mixed_c4.md" and t256 == pytest.approx(4 * t64, rel=1e-9)
    # workloads without a capture report none
    assert bench.profile_traffic("c1", "MIXED", 1.0) == (None, None)
    assert bench.profile_traffic("c4", "FP64", 1.0) == (None, None)


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def test_clock_record_marks_an_unsampled_region():
    c = bench.ClockSampler(0)
    c.proc = _FakeProc()
    out = c.stop()
    assert out["reasons"] == ["unsampled"] and out["samples"] == 0 and out["sm_mhz"] is None
    c = bench.ClockSampler(0)   # nvidia-smi could not be started
    assert c.stop()["reasons"] == ["unsampled"]


def test_clock_record_reports_median_clock_and_throttle_reasons():
    c = bench.ClockSampler(0)
    c.proc = _FakeProc()
    c.rows = [["2070", "2070", "900.1", "Not Active", "Not Active", "Not Active", "Not Active"],
              ["1980", "2070", "1380.0", "Not Active", "Not Active", "Not Active", "Active"],
              ["2070", "2070", "1100.5", "Not Active", "Not Active", "Not Active", "Not Active"]]
    out = c.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]


def test_timed_windows_stay_inside_the_bounded_steps():
    # C2 runs away from about step 280 and C4's first plates from about 225
    # under the reference's failure model; C1 stays bounded over its 1,000 steps
    assert bench.STEP_WINDOW["c2"] <= 280 and bench.STEP_WINDOW["c4"] <= 225
    assert bench.STEP_WINDOW["c1"] >= 1000
    assert set(bench.WINDOW_REASON) == set(bench.STEP_WINDOW)


def test_fc1_cpu_baseline_reproduces_the_reference_sif():
    """The FC 1 bench's CPU leg (oracle set-up and assembly, SuperLU, FC 1
    oracle; no product code) on the 31 x 31 plate: its KI for the loaded
    increment equals the reference's."""
    from conftest import case_cmd, golden
    t, ki = bench.cpu_sample_fc1(case_cmd("pe31", "pe31_fc1"))
    ref = golden("pe31_fc1")["crack_rows"][1, 0, 3]
    assert t > 0 and abs(ki - ref) <= 1e-10 * abs(ref)
