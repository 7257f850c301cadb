"""bench.py's CPU-side pieces: the roofline traffic it reports comes from the
committed ncu summaries (per fact row for the star kernel, per shared-scan
byte for the batch kernel), and its command line parses."""
import os
import subprocess
import sys

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_star_kernel_traffic_is_committed():
    tr = bench.committed_traffic(2)
    assert tr is not None
    # three int32 columns streamed (12 B per fact row) and the two late metric
    # columns gathered at the surviving rows' sectors: below the 20 B the five
    # columns would take
    assert 12.0 < tr["dram_bytes_per_row"] < 20.0
    assert "star_plan_kernel_config2.md" in tr["source"]
    # the String-dimension query runs the same kernel over the same fact columns
    assert bench.committed_traffic(5) == tr
    # configs 0 and 1 have captures of their own
    assert 8.0 < bench.committed_traffic(1)["dram_bytes_per_row"] < 12.0
    assert 12.0 < bench.committed_traffic(0)["dram_bytes_per_row"] < 16.0


def test_batch_kernel_traffic_is_committed():
    tr = bench.committed_traffic(3)
    assert tr is not None
    # the shared scan reads the union of the queries' columns once
    assert 1.0 <= tr["dram_bytes_per_scan_byte"] < 1.05
    assert "mbatch_kernel_config3.md" in tr["source"]


def test_unknown_workload_has_no_committed_traffic():
    assert bench.committed_traffic(4) is None


def test_command_line_parses():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--config"):
        assert flag in r.stdout


def test_reference_arm_prints_its_contract_line():
    """--impl reference times the reference's generated CPU path (the oracle
    port) on a bounded sample and prints one JSON line with the keys the
    comparison reads; here on a tiny config-0 sample."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "0",
                        "--cpu-sample-rows", "200000", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "fact rows/s" and d["unit"] == "rows/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("config 0")
