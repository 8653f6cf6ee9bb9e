"""The bindings INTEGRATION.md shows a maintainer of the reference are real
code: its C++ replacement of the reference's solver block compiles against
include/ns3d_capi.h and links against the CUDA library, and its Python
(ctypes) example runs as written (on the CPU oracle, which implements the
same header)."""
import os
import re
import subprocess

import numpy as np

from ns3d_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _blocks(lang):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```%s\n(.*?)```" % lang, text, re.S)


# what the snippet takes from the reference's main: its InputParams fields
# (src/navierstokes3D.cxx) and the output stem
CPP_FRAME = r"""
#include <cstdio>
#include <string>
#include <vector>
%(include)s
struct InputParams {
    std::string image, method;
    double dx, dy, dz, mu, rho, p0, gradp, alpha, beta, vsolvertol, psolvertol, pcsolvertol, simpletol, deltaRMR;
    int maxitsolver, maxitSIMPLE, N1, N2, save_step, porevalue, direction, border;
};
int run(const InputParams &p, const std::string &stem) {
%(body)s
    return 0;
}
int main() { return 0; }
"""


def test_cpp_replacement_compiles_and_links(gpulib, tmp_path):
    block = _blocks("cpp")[0]
    include = "\n".join(l for l in block.splitlines() if l.startswith("#include"))
    body = "\n".join(l for l in block.splitlines() if not l.startswith("#include"))
    src = tmp_path / "replacement.cpp"
    src.write_text(CPP_FRAME % {"include": include, "body": body})
    lib_dir = os.path.join(ROOT, "ns3d_gb300", "_lib")
    out = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                          str(tmp_path / "replacement"), "-L", lib_dir, "-lns3d_gb300",
                          "-Wl,--allow-shlib-undefined"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


def test_python_example_runs(oracle):
    block = _blocks("python")[0]
    img_c_order, _ = synth.rsa_spheres((14, 10, 12), 2, 0.65, seed=7)
    from tests.conftest import ORACLE_LIB
    code = block.replace('"ns3d_gb300/_lib/libns3d_gb300.so"', repr(ORACLE_LIB))
    scope = {"img_c_order": img_c_order}
    exec(compile(code, "INTEGRATION.md", "exec"), scope)
    r = scope["r"]
    assert r.iterations > 0 and np.isfinite(r.K) and r.K > 0
    assert [a.shape[0] for a in (scope["p"], scope["u"], scope["v"], scope["w"])] == \
        [scope["s"].sizes.np, scope["s"].sizes.nu, scope["s"].sizes.nv, scope["s"].sizes.nw]
