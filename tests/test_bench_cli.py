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
