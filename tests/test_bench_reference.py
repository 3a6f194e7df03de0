"""bench.py's reference arm on the CPU: the oracle (the reference's
algorithm restated, brute-force triangle loops) timed on a bounded sample of
a workload prints one JSON line with the contract's keys, the arm's `impl`
and a `cpu_baseline` describing the run."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--workload", "relief_hall", "--steps", "1", "--warmup", "3",
                        "--cpu-rays", "2"], capture_output=True, text=True, timeout=600,
                       cwd=str(ROOT))
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "ray-bounce segments/s"
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["config"]["workload"] == "relief-hall-20k-stereo"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
