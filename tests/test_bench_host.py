"""Host logic of bench.py on CPU: the clock sampler's summary of the
nvidia-smi lines taken inside the timed region (after the mark), with a
stand-in for the sampler process. No GPU."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def poll(self):
        return None


def _sampler(tmp_path, lines, skip):
    cs = bench.ClockSampler(0)
    path = tmp_path / "clocks.csv"
    path.write_text("".join(line + "\n" for line in lines))
    cs.path, cs.proc, cs.skip = str(path), _Proc(), skip
    return cs


ROW = "0, {sm}, 2070, {pw}, 0x0, Not Active, Not Active, {sw_thermal}, {power_cap}"


def test_clock_summary_keeps_the_lines_after_the_mark(tmp_path):
    lines = [ROW.format(sm=1005, pw=120.0, sw_thermal="Active", power_cap="Not Active"),  # warm-up, idle
             ROW.format(sm=2070, pw=900.0, sw_thermal="Not Active", power_cap="Active"),
             ROW.format(sm=2070, pw=950.0, sw_thermal="Not Active", power_cap="Not Active"),
             ROW.format(sm=2055, pw=940.0, sw_thermal="Not Active", power_cap="Not Active")]
    r = _sampler(tmp_path, lines, skip=1).stop()
    assert r["samples"] == 3
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]  # the warm-up line's reason is not counted


def test_clock_summary_falls_back_to_all_lines_when_none_follow_the_mark(tmp_path):
    lines = [ROW.format(sm=2070, pw=900.0, sw_thermal="Not Active", power_cap="Not Active")] * 2
    r = _sampler(tmp_path, lines, skip=2).stop()
    assert r["samples"] == 2 and r["reasons"] == []


def test_clock_summary_ignores_malformed_lines(tmp_path):
    lines = ["garbage", ROW.format(sm=2070, pw=900.0, sw_thermal="Not Active", power_cap="Not Active"),
             "0, [N/A], 2070, 1.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    r = _sampler(tmp_path, lines, skip=0).stop()
    assert r["samples"] == 1 and r["sm_mhz"] == 2070.0
