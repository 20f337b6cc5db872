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


def _traffic_csv(path, launches):
    """An ncu --csv metrics log with the two DRAM counters per launch."""
    rows = ['"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size",'
            '"Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"']
    for i, (rd, wr) in enumerate(launches):
        for name, unit, val in (("dram__bytes_read.sum", "Mbyte", rd), ("dram__bytes_write.sum", "Kbyte", wr)):
            rows.append(f'"{i}","1","python3","h","void k_mf_points<float, 11, 1, 8, 3>(JacSrc<float>)","1","7",'
                        f'"(256, 1, 1)","(2909, 1, 1)","0","10.3","Command line profiler metrics","{name}",'
                        f'"{unit}","{val}"')
    path.write_text("\n".join(rows) + "\n")


def test_record_traffic_skips_launches_of_converged_solves(tmp_path, monkeypatch):
    """Launches after a PCG solve converged return at once (a few KB of DRAM
    traffic): the per-launch figure is the mean of the launches that ran an
    iteration, keyed by the pass's sources."""
    csv = tmp_path / "traffic.csv"
    _traffic_csv(csv, [(0.011776, 0.0), (140.0, 3000.0), (0.011520, 0.0), (142.0, 5000.0)])
    out = tmp_path / "ncu_traffic.json"
    monkeypatch.setattr(bench, "TRAFFIC_FILE", str(out))
    args = bench.argparse.Namespace(record_traffic=str(csv), workload="radial2000", scale=1.0)
    bench.record_traffic(args)
    import json

    e = json.load(open(out))["entries"][0]
    assert e["launches_captured"] == 2
    assert e["dram_bytes_per_launch"] == int((140e6 + 3e6 + 142e6 + 5e6) / 2)
    assert e["sources_sha"] == bench.sources_sha(bench.POINT_PASS_SOURCES)
    traffic, src = bench.ncu_traffic("pcg_points", "radial2000", 1.0)
    assert traffic == e["dram_bytes_per_launch"] and "ncu" in src


def test_traffic_of_changed_sources_is_not_reported(tmp_path, monkeypatch):
    import json

    out = tmp_path / "ncu_traffic.json"
    out.write_text(json.dumps({"entries": [{"phase": "pcg_points", "workload": "radial2000", "scale": 1.0,
                                            "dram_bytes_per_launch": 1, "sources": bench.POINT_PASS_SOURCES,
                                            "sources_sha": "0000000000000000"}]}))
    monkeypatch.setattr(bench, "TRAFFIC_FILE", str(out))
    traffic, src = bench.ncu_traffic("pcg_points", "radial2000", 1.0)
    assert traffic is None and "changed" in src
