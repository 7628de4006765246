"""The benchmark's reference arm on the host cores (no GPU): one JSON line with the contract's keys,
its CPU baseline describing the run and a zero-copy e2e figure equal to its value."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == "probe-rays/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same config object as the GPU arm's line, so the two lines compare as one workload
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == dict(bench.WORKLOAD, l2="flushed between steps (256 MiB write)", parallelism="single GPU")
