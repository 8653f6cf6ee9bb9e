"""The NS3D program (`ns3d_gb300/_lib/NS3D <file.ini>`, the reference's argv
contract, src/navierstokes3D.cxx:480-545): it reads the ini and the .vti
image, solves, and writes the INFO/RES logs and the P/Vx/Vy/Vz/V images the
reference writes (src/NSBase.cxx:107-123,330-476); its K and fields equal
those of the same case solved through the library."""
import re
import subprocess

import numpy as np
import pytest

import ns3d_gb300 as ns
from ns3d_gb300 import synth

pytestmark = pytest.mark.gpu

INI = """# permeability of a sphere pack
input = pack.vti
pressurefield = none   # start from the linear pressure profile
dx = 1e-6
mu = 1e-3
rho = 1
p0 = 1
gradp = {gradp}
alpha = 0.5
vsolvertol = 1e-8
psolvertol = 1e-8
pcsolvertol = 1e-8
simpletol = 1e-5
maxitsolver = 500
maxitSIMPLE = 40
method = {method}
direction = 1
"""


@pytest.mark.parametrize("method", ["SIMPLEC", "IDEAL"])
def test_ns3d_program_outputs_match_the_library(gpulib, tmp_path, method):
    img, _ = synth.rsa_spheres((20, 18, 16), 3, 0.6, seed=31)
    ns.write_vti_u8(tmp_path / "pack.vti", img)
    (tmp_path / "case.ini").write_text(INI.format(gradp=1.0 / (20 * 1e-6), method=method))
    run = subprocess.run([ns.EXE_PATH, "case.ini"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr
    for name in ("INFO-1-pack.log", "RES-1-pack.csv", "P-1-pack.vti", "Vx-1-pack.vti", "Vy-1-pack.vti",
                 "Vz-1-pack.vti", "V-1-pack.vti"):
        assert (tmp_path / name).exists(), name
    # the same case through the library
    prm, files = ns.read_ini(tmp_path / "case.ini")
    assert files["input"] == "pack.vti"
    s = ns.open_solver(prm, img)
    r = s.solve()
    info = (tmp_path / "INFO-1-pack.log").read_text()
    ks = [float(x) for x in re.findall(r"^Permeability K \(m²\): (\S+)$", info, re.M)]
    assert ks and abs(ks[-1] - r.K) <= 1e-14 * abs(r.K)   # the log prints 15 digits
    p, u, v, w, va = s.field_images()
    assert np.array_equal(ns.read_vti_f64(tmp_path / "P-1-pack.vti"), p)
    assert np.array_equal(ns.read_vti_f64(tmp_path / "Vx-1-pack.vti"), u)
    assert np.array_equal(ns.read_vti_f64(tmp_path / "V-1-pack.vti"), va)
    if method == "SIMPLEC":
        rows = (tmp_path / "RES-1-pack.csv").read_text().splitlines()
        assert rows[0].startswith("iteration") and len(rows) >= 2
        assert float(rows[-1].split(",")[4]) == pytest.approx(r.K, rel=1e-5)   # K column, 6 digits
    s.close()


def test_ns3d_program_usage_and_input_error(gpulib, tmp_path):
    assert subprocess.run([ns.EXE_PATH, "-h"], capture_output=True).returncode == 0
    (tmp_path / "bad.ini").write_text("input = missing.vti\n")
    assert subprocess.run([ns.EXE_PATH, "bad.ini"], cwd=tmp_path, capture_output=True).returncode == 1
