"""bench.py's output contract, checked on the CPU through its reference arm (the oracle's element loop on the host
cores): one JSON line with the metric, the reference's CPU baseline and an end-to-end figure with no device
copies, so that both arms can be compared line by line."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "poisson-8",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "GDoF/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == "poisson-8^3-p4"
    # the same config object as the GPU arm's line for this workload (the full workload, not a sample of it)
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.workload_config(bench.CONFIGS["poisson-8"], 29791)
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
