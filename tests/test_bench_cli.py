"""The benchmark's reference arm on any machine: the reference's own solver
cannot be built and its CPU restatement cannot finish complete solves of the
serving stream inside one run, so `bench.py --impl reference` prints one JSON
line saying why and exits 0 (nothing is modelled or extrapolated)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_unavailable_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=120,
                         env=dict(os.environ, WORLD_SIZE="1", RANK="0"))
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["unavailable"]
    assert rec["metric"].startswith("permeability solves/sec")
    assert "5 complete solves" in rec["unavailable"]
