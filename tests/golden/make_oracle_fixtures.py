"""Run the CPU oracle on the full-size seeded workloads and record its
results as parity fixtures (tests/golden/oracle_<case>_<method>.json plus
the RES/INFO logs, gzip-compressed, under tests/golden/oracle_logs/).

Cases (ns3d_gb300/workloads.py): sphere64 (64^3 RSA spheres r = 6,
porosity ~0.55, seed 0, SIMPLEC) and sphere128 (128^3 RSA spheres r = 8,
porosity ~0.5, seed 1; SIMPLEC, SIMPLER, SIMPLERR, IDEAL), all solved to
convergence (RMR < 1e-6, BiCGSTAB tolerances 1e-8).

Each record holds the image's SHA-256 and porosity, every scalar of the final
ns3d_result (K and the others as 17-digit reprs), the outer and BiCGSTAB
iteration counts, per-field L2 norms and the SHA-256 of each compacted
field's bytes (p, u, v, w in the solver's row numbering), and the SHA-256 of
the RES and INFO logs with the wall-clock line ("... terminated in N
iteration and S seconds") removed.  The CUDA path follows the oracle's
arithmetic bit for bit, so the GPU tests compare these hashes exactly.

The oracle uses no transcendental function and is built with
-ffp-contract=off, so its results are the same bits on any IEEE-754 host
(x86-64 or Arm); the records can be made on whichever host has the cores.

The oracle is test infrastructure: this script runs on the CPU only.
Usage: python tests/golden/make_oracle_fixtures.py [--out DIR] [case[:method]] ...
(no case: every case; a sphere128 solve takes 5-90 minutes by method and
host).  NS3D_ORACLE_LIB may name a private copy of the oracle library, so
that a rebuild of oracle/_build during a long run does not touch the one in
use.
"""
import gzip
import hashlib
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ns3d_gb300 import capi, synth, workloads  # noqa: E402

OUT = HERE
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libns3d_oracle.so")


def strip_clock(text):
    """Log text without the wall-clock line of the outer drivers."""
    return "".join(l for l in text.splitlines(True) if " terminated in " not in l)


def sha(b):
    return hashlib.sha256(b).hexdigest()


def fixture_path(case, method):
    return os.path.join(OUT, "oracle_%s_%s.json" % (case, method))


def run_case(lib, case, method, img, info):
    spec = workloads.CASES[case]
    prm = workloads.solve_params(capi, lib, img.shape[spec["direction"] - 1], method, spec["direction"])
    s = capi.Solver(lib, prm, synth.to_raw(img), img.shape)
    tmp = tempfile.mkdtemp(prefix="ns3d_fixture_")
    stem = "%s_%s" % (case, method)
    s.set_output(tmp, stem, False)
    t = time.perf_counter()
    r = s.solve()
    seconds = time.perf_counter() - t
    fields = s.fields()
    sizes = dict(np=s.sizes.np, nu=s.sizes.nu, nv=s.sizes.nv, nw=s.sizes.nw)
    s.close()
    d = str(spec["direction"])
    res = strip_clock(open(os.path.join(tmp, "RES-%s-%s.csv" % (d, stem))).read())
    inf = strip_clock(open(os.path.join(tmp, "INFO-%s-%s.log" % (d, stem))).read())
    logs = os.path.join(OUT, "oracle_logs")
    os.makedirs(logs, exist_ok=True)
    for kind, text in (("RES", res), ("INFO", inf)):
        with gzip.GzipFile(os.path.join(logs, "%s_%s.%s.gz" % (case, method, kind)), "wb", mtime=0) as f:
            f.write(text.encode())
    result = {}
    for name, _ in capi.Result._fields_:
        if name == "seconds":
            continue
        v = getattr(r, name)
        result[name] = repr(float(v)) if isinstance(v, float) else int(v)
    rec = {
        "case": case, "method": method,
        "image": {"shape": list(img.shape), "sha256": workloads.image_sha256(img), "porosity": info["porosity"],
                  "generator": {k: v for k, v in info.items() if k != "porosity"}},
        "params": {k: (repr(v) if isinstance(v, float) else v) for k, v in prm.as_dict().items()},
        "sizes": sizes,
        "result": result,
        "fields": {n: {"n": int(a.size), "l2": repr(float(np.linalg.norm(a))), "sha256": workloads.field_sha256(a)}
                   for n, a in zip(("p", "u", "v", "w"), fields)},
        "res_sha256": sha(res.encode()), "info_sha256": sha(inf.encode()),
        "res_lines": len(res.splitlines()), "info_lines": len(inf.splitlines()),
        "oracle": {"host": platform.machine(),
                   "threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                   "seconds": seconds},
    }
    with open(fixture_path(case, method), "w") as f:
        json.dump(rec, f, indent=1)
    print("%s %s: K=%s outer=%d krylov=%d %.0f s" % (case, method, result["K"], r.iterations,
                                                     r.krylov_iterations, seconds), flush=True)


def main(argv):
    global OUT
    if argv[:1] == ["--out"]:
        OUT = os.path.abspath(argv[1])
        argv = argv[2:]
    os.makedirs(OUT, exist_ok=True)
    lib_path = os.environ.get("NS3D_ORACLE_LIB")
    if not lib_path:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        lib_path = ORACLE_LIB
    lib = capi.load(lib_path)
    wanted = []
    for a in (argv or list(workloads.CASES)):
        case, _, method = a.partition(":")
        for m in ([method] if method else workloads.CASES[case]["methods"]):
            wanted.append((case, m))
    images = {}
    for case, method in wanted:
        if case not in images:
            images[case] = workloads.CASES[case]["image"]()
        img, info = images[case]
        run_case(lib, case, method, img, info)


if __name__ == "__main__":
    main(sys.argv[1:])
