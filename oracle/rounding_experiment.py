"""How much does a solve's trajectory depend on rounding alone?

The reference's published results were produced with Eigen, whose SIMD
reduction order cannot be reproduced.  This experiment solves the
reference's own cases with the CPU oracle under three roundings of the
BiCGSTAB arithmetic (environment variable NS3D_ORACLE_ARITH of the oracle):
  fixed     the documented order the CUDA path follows (chunked lanes and
            trees, fused multiply-adds where written)
  serial    products rounded before each add, one accumulator per dot product
  packet4   as serial, dot products with 4 interleaved accumulators

Case 1, the README table (its tests/compare_algorithms.ini on the 64^3
sphere lattice data/spheres_64.vti, four methods): per method and rounding,
the outer-iteration count at convergence and K.  If a method's count moves
with the rounding alone while K stays put, a count that differs from the
published one is a rounding effect, not an error of the restatement.

Case 2, the golden run (tests/test_spheres.ini on the 128^3 lattice,
SIMPLEC, 30 outer iterations, pressure-correction tolerance 1e-3): the K of
every iteration under each rounding and the largest relative spread between
roundings per iteration.  With `--golden-k FILE`
(tests/golden/reference_runs.json) the reference's own 15-digit K lines are
put beside them.

The oracle is test infrastructure; this script runs it on the CPU only.
Usage: python oracle/rounding_experiment.py [out.json] [--golden-k FILE]
(about a minute per 64^3 solve and five per golden run on 8 cores; each
rounding runs in its own process because the oracle reads the variable when
a solver opens).
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import json, sys
sys.path.insert(0, %(root)r)
from ns3d_gb300 import capi, synth
lib = capi.load(%(lib)r)
img = synth.sphere_lattice(64, 8, 3)
p = capi.default_params(lib, dx=2e-6, dy=-1.0, dz=-1.0, mu=1e-3, rho=1e3, p0=1e5, gradp=1e2, alpha=0.8, beta=1.0,
                        vsolvertol=1e-5, psolvertol=1e-6, pcsolvertol=1e-3, simpletol=1e-4, maxitsolver=500,
                        maxitSIMPLE=200, N1=2, N2=2, porevalue=0, direction=1, border=0, method=%(method)r)
s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
r = s.solve()
print(json.dumps({"K": r.K, "outer_iterations": int(r.iterations), "converged": int(r.converged),
                  "RMR": r.RMR}))
"""

GOLDEN_CHILD = r"""
import json, os, sys, tempfile
sys.path.insert(0, %(root)r)
from ns3d_gb300 import capi, synth
lib = capi.load(%(lib)r)
img = synth.sphere_lattice(128, 12, 5)
p = capi.default_params(lib, dx=2e-6, dy=-1.0, dz=-1.0, mu=1e-3, rho=1e3, p0=1e5, gradp=1e2, alpha=0.8, beta=1.0,
                        vsolvertol=1e-5, psolvertol=1e-6, pcsolvertol=1e-3, simpletol=1e-4, maxitsolver=500,
                        maxitSIMPLE=30, N1=2, N2=2, porevalue=0, direction=1, border=0, method="SIMPLEC")
s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
d = tempfile.mkdtemp()
s.set_output(d, "g", False)
r = s.solve()
ks = [float(l.split(":")[1]) for l in open(os.path.join(d, "INFO-1-g.log")) if l.startswith("Permeability K")]
print(json.dumps({"K_per_iteration": ks}))
"""

MODES = ("fixed", "serial", "packet4")


def child(code, mode):
    env = dict(os.environ, NS3D_ORACLE_ARITH=mode)
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    return json.loads(p.stdout.strip().splitlines()[-1])


def main():
    args = sys.argv[1:]
    golden_k = None
    if "--golden-k" in args:
        i = args.index("--golden-k")
        golden_k = [float(x) for x in json.load(open(args[i + 1]))["info_K_per_iteration"]]
        del args[i:i + 2]
    out = args[0] if args else os.path.join(HERE, "rounding_experiment.json")
    lib = os.environ.get("NS3D_ORACLE_LIB", os.path.join(HERE, "_build", "libns3d_oracle.so"))
    if not os.path.exists(lib):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    published = {"SIMPLEC": (3.28386e-12, 48), "SIMPLER": (3.28382e-12, 42), "SIMPLERR": (3.28175e-12, 23),
                 "IDEAL": (3.28212e-12, 19)}
    res = {"case": "README 64^3 compare_algorithms table (sphere lattice spacing 8 radius 3), oracle",
           "published": {m: {"K": k, "outer_iterations": it} for m, (k, it) in published.items()}, "runs": {}}
    for method in published:
        for mode in MODES:
            r = child(CHILD % {"root": ROOT, "lib": lib, "method": method}, mode)
            r["K_rel_diff_vs_published"] = abs(r["K"] - published[method][0]) / published[method][0]
            res["runs"].setdefault(method, {})[mode] = r
            print(method, mode, r, flush=True)
    runs = {}
    for mode in MODES:
        runs[mode] = child(GOLDEN_CHILD % {"root": ROOT, "lib": lib}, mode)["K_per_iteration"]
        print("golden", mode, runs[mode][-1], flush=True)
    spread = [max(abs(runs[a][i] - runs[b][i]) / abs(runs["fixed"][i]) for a in runs for b in runs)
              for i in range(len(runs["fixed"]))]
    g = {"case": "reference tests/test_spheres.ini on the 128^3 lattice, SIMPLEC, 30 iterations, oracle",
         "K_per_iteration": runs, "max_rel_spread_between_roundings": spread}
    if golden_k:
        g["reference_K_per_iteration"] = golden_k
        g["max_rel_diff_to_reference"] = {m: [abs(k - gk) / gk for k, gk in zip(ks, golden_k)]
                                          for m, ks in runs.items()}
    res["golden128"] = g
    with open(out, "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
