"""The benchmark's reference arm (`bench.py --impl reference`) runs on the
host cores only: one JSON line with the keys the measurement contract asks
for, on the same metric and workload as the GPU arm."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_reference_arm_json_line():
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "4"))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in r, key
    assert r["metric"] == "Fock builds/s (J+K)" and r["unit"] == "builds/s"
    assert r["value"] > 0 and r["higher_is_better"] is True
    assert r["cpu_baseline"]["value"] == r["value"] and r["cpu_baseline"]["kind"] in ("port", "reference")
    assert r["e2e"]["value"] == r["value"] and r["e2e"]["h2d_bytes_per_step"] == 0
    assert "Kr" in r["config"]["workload"]
