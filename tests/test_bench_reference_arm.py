"""The reference arm of bench.py (the CPU solver the GPU path is compared
with) runs without a GPU: its JSON line carries the contract's keys, and a
bounded CPU-baseline sample steps on to its time target."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "c0",
                          "--steps", "1", "--warmup", "0", "--ref-sample", "2"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] == line["value"]


def test_cpu_baseline_time_target():
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "ard-simulator_gb300"))
    import bench
    cfg = bench.workload("c0", sim_steps=40)
    cb = bench.cpu_baseline(cfg, 1, 0.5)
    steps = int(cb["sample"].split()[0])
    assert 1 <= steps <= 39
    assert cb["value"] > 0 and cb["unit"] == "Gcell-steps/s"
