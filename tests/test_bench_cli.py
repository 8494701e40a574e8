"""bench.py's command line parses (no GPU): the driver calls it with --gpus/--steps/--warmup
and --impl reference, and the profiling recipes with --workload/--fmax."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_help_parses():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--fmax", "--precision"):
        assert opt in r.stdout


def test_reference_arm_line_on_cpu():
    """`--impl reference` runs the reference's CPU algorithm on the host cores (no GPU): one JSON
    line with the arm's fields (impl, the metric and its unit, a cpu_baseline describing the run
    and an e2e with no host-device bytes), here on the one-shot split-step workload."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "split1",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "shot*omega*depth-steps/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] >= 3
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
