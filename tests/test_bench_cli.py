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


def test_oracle_reports_phase_times(oracle):
    """The CPU baseline's per-phase wall times (assembly, BiCGSTAB,
    corrections, diagnostics) cover the solve and are reset by each solve."""
    import ctypes as C
    import time
    from helpers import params, solver
    from ns3d_gb300 import synth
    img, _ = synth.rsa_spheres((16, 12, 14), 2, 0.6, seed=5)
    s = solver(oracle, img, params(oracle, method="IDEAL", maxitSIMPLE=20))
    for _ in range(2):
        t = time.perf_counter()
        s.solve()
        dt = time.perf_counter() - t
        ph = (C.c_double * 4)()
        assert oracle.ns3d_oracle_phase_seconds(ph) == 0
        assert all(x > 0 for x in ph) and sum(ph) <= dt
    s.close()
