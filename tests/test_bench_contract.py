"""bench.py's reference arm on the CPU: one JSON line with the GPU arm's metric,
unit and workload, the oracle's timing as value, a cpu_baseline describing the
run and an e2e block without host-device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    sys.path.insert(0, ROOT)
    import bench
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["config"]["workload"] == bench.CONFIG["workload"]
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_roofline_traffic_covers_the_whole_apply():
    """The headline roofline's traffic is the DRAM bytes of one apply, both
    kernels (as its achieved bandwidth is), from the committed ncu summary;
    the main kernel's own bytes and launch share are reported beside it."""
    sys.path.insert(0, ROOT)
    import bench
    step, main, share = bench.profiled_traffic(os.path.join(ROOT, "profiles", "dg_trace_const_q3_64cube_f64.json"))
    with open(os.path.join(ROOT, "profiles", "dg_trace_const_q3_64cube_f64.json")) as f:
        d = json.load(f)
    t = d["trace_kernel"]
    assert main == d["dram_read"] + d["dram_write"]
    assert step == main + t["dram_read"] + t["dram_write"]
    assert 0.5 < share < 1.0
    assert bench.profiled_traffic(os.path.join(ROOT, "profiles", "missing.json")) == (None, None, None)
