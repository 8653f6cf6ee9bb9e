"""Compare the CPU oracle with the reference's whole golden run and record
the comparison (tests/golden/oracle_lattice128_golden.json) plus the
oracle's own logs of that run (tests/golden/oracle_logs/lattice128_golden.*.gz).

The golden run is the reference's tests/test_spheres.ini on its
data/spheres_128.vti (a 128^3 regular sphere lattice, regenerated here byte
for byte by synth.sphere_lattice(128, 12, 5)): SIMPLEC, 30 outer iterations,
a field snapshot at iteration 20 (save_step 20).  Its outputs are the
reference's tests/results/RES-1-spheres_128.csv (30 rows, 6 digits),
INFO-1-spheres_128.log (15-digit K per iteration) and the Float64 fields
{P,Vx,Vy,Vz}-1-spheres_128{-SAVE-1,}.vti.

Recorded: the oracle's 30 RES rows and K lines (in its logs), the relative
L2 difference of each oracle field against the golden field (over the whole
image, 0 at solid voxels in both), and the SHA-256 of the oracle's field
images, which the GPU test compares bit for bit.

Needs the reference checkout (read-only).  Usage:
  python tests/golden/make_golden_run.py <reference root>
(or set NS3D_REFERENCE_ROOT).  About five minutes on 8 cores.
"""
import gzip
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from ns3d_gb300 import capi, synth  # noqa: E402
import vtiutil  # noqa: E402

ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libns3d_oracle.so")
FIELDS = ("P", "Vx", "Vy", "Vz")


def strip_clock(text):
    return "".join(l for l in text.splitlines(True) if " terminated in " not in l)


def golden_params(lib):
    """tests/test_spheres.ini of the reference, as ns3d_params."""
    return capi.default_params(lib, dx=2e-6, dy=-1, dz=-1, mu=1e-3, rho=1e3, p0=1e5, gradp=1e2, alpha=0.8,
                               beta=1.0, vsolvertol=1e-5, psolvertol=1e-6, pcsolvertol=1e-3, simpletol=1e-4,
                               deltaRMR=1e-4, maxitsolver=500, maxitSIMPLE=30, N1=2, N2=2, save_step=20,
                               porevalue=0, direction=1, border=0, method="SIMPLEC")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def main(argv):
    ref = argv[0] if argv else os.environ.get("NS3D_REFERENCE_ROOT")
    if not ref:
        sys.exit("usage: make_golden_run.py <reference root> (or NS3D_REFERENCE_ROOT)")
    lib_path = os.environ.get("NS3D_ORACLE_LIB")
    if not lib_path:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        lib_path = ORACLE_LIB
    lib = capi.load(lib_path)
    img = synth.sphere_lattice(128, 12, 5)
    raw = synth.to_raw(img)
    # the snapshot of iteration 20 is the state after a 21-iteration run (the
    # reference saves it at the end of iteration 20; nothing after that point
    # of the iteration changes the fields)
    snapshots = {}
    for snap, outer in (("iteration_20", 21), ("iteration_30", 30)):
        prm = golden_params(lib)
        prm.maxitSIMPLE = outer
        s = capi.Solver(lib, prm, raw, img.shape)
        tmp = tempfile.mkdtemp(prefix="ns3d_golden_")
        s.set_output(tmp, "spheres_128", False)
        r = s.solve()
        snapshots[snap] = (s.field_images(), r, tmp)
        s.close()
    images, r, tmp = snapshots["iteration_30"]
    res = strip_clock(open(os.path.join(tmp, "RES-1-spheres_128.csv")).read())
    inf = strip_clock(open(os.path.join(tmp, "INFO-1-spheres_128.log")).read())
    logs = os.path.join(HERE, "oracle_logs")
    os.makedirs(logs, exist_ok=True)
    for kind, text in (("RES", res), ("INFO", inf)):
        with gzip.GzipFile(os.path.join(logs, "lattice128_golden.%s.gz" % kind), "wb", mtime=0) as f:
            f.write(text.encode())
    fields = {}
    for snap, suffix in (("iteration_30", ""), ("iteration_20", "-SAVE-1")):
        for name, mine in zip(FIELDS, snapshots[snap][0][:4]):
            fn = "%s-1-spheres_128%s.vti" % (name, suffix)
            gold, _ = vtiutil.read_vti(os.path.join(ref, "tests", "results", fn))
            assert mine.shape == gold.shape, (fn, mine.shape, gold.shape)
            fields.setdefault(snap, {})[name] = {"rel_l2": rel_l2(mine, gold), "shape": list(gold.shape),
                                                 "golden_l2": float(np.linalg.norm(gold)),
                                                 "oracle_l2": float(np.linalg.norm(mine))}
    names = ("p", "u", "v", "w", "v_faces")
    out = {
        "case": "reference tests/test_spheres.ini on data/spheres_128.vti (regenerated), SIMPLEC, 30 iterations",
        "oracle_result": {"K": repr(r.K), "iterations": int(r.iterations), "RMR": repr(r.RMR)},
        "field_rel_l2_vs_golden": fields,
        "oracle_field_images_sha256": {n: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
                                       for n, a in zip(names, images)},
        "res_sha256": hashlib.sha256(res.encode()).hexdigest(),
        "info_sha256": hashlib.sha256(inf.encode()).hexdigest(),
    }
    with open(os.path.join(HERE, "oracle_lattice128_golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(fields, indent=1))


if __name__ == "__main__":
    main(sys.argv[1:])
