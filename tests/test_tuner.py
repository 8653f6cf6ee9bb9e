"""Host logic of the merged-set grid autotuner (GridTuner): round-robin
exploration, the pick by mean time per row-iteration, classes, the switch
and reset.  Built from the library's own tuner.cpp with g++; no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_grid_tuner_logic(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    exe = str(tmp_path / "tuner_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "tuner_check.cpp"),
                    os.path.join(ROOT, "ns3d_gb300", "csrc", "tuner.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], stdout=subprocess.PIPE, text=True)
    assert out.returncode == 0 and out.stdout.strip().endswith("OK"), out.stdout
