"""Generate tests/golden/reference_runs.json from the reference's own
published results (run once where the reference checkout is available;
the checkout's root is the first argument, or NS3D_REFERENCE_ROOT).

Sources (paths inside the reference project):
  tests/results/RES-1-spheres_128.csv   per-iteration RES rows of test_spheres.ini
  tests/results/INFO-1-spheres_128.log  node counts, porosity, 15-digit K values
  README.md                              the 64^3 compare_algorithms table
  tests/test_spheres.ini, tests/compare_algorithms.ini   the run parameters
  data/spheres_64.vti, data/spheres_128.vti              sha256 of the voxel data
"""
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import vtiutil  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NS3D_REFERENCE_ROOT")


def ini(path):
    out = {}
    for line in open(path):
        line = line.split("#")[0].strip()
        if "=" in line:
            k, v = [s.strip() for s in line.split("=", 1)]
            out[k] = v
    return out


def main():
    if not REF:
        sys.exit("usage: make_golden.py <reference root> (or set NS3D_REFERENCE_ROOT)")
    res_lines = open(os.path.join(REF, "tests/results/RES-1-spheres_128.csv")).read().splitlines()
    header = res_lines[0]
    rows = []
    for l in res_lines[1:]:
        f = [x.strip() for x in l.split(",")]
        rows.append([int(f[0])] + [float(x) for x in f[1:10]] + [int(x) for x in f[10:13]] + [f[13]])
    info = open(os.path.join(REF, "tests/results/INFO-1-spheres_128.log")).read().splitlines()
    counts = {}
    for key, name in (("np", "pressure"), ("nu", "u velocity"), ("nv", "v velocity"), ("nw", "w velocity")):
        counts[key] = int([l for l in info if l.startswith("Nodes for the %s field" % name)][0].split(":")[1])
    porosity_line = [l for l in info if l.startswith("Porosity:")][0]
    initial_k = [l for l in info if l.startswith("Initial Permeability")][0].split(":")[1].strip()
    k_lines = [l.split(":")[1].strip() for l in info if l.startswith("Permeability K")]
    solves = [l for l in info if l.startswith("Solving for")]
    readme = open(os.path.join(REF, "README.md")).read()
    table = {}
    for m in re.finditer(r"^(SIMPLEC|SIMPLER|SIMPLERR|IDEAL)\s+([0-9.e+-]+)\s+(\d+)\s+([0-9.]+)\s+(\w+)", readme, re.M):
        table[m.group(1)] = {"K": float(m.group(2)), "iterations": int(m.group(3)), "seconds": float(m.group(4))}
    images = {}
    for name in ("spheres_64.vti", "spheres_128.vti"):
        a, _ = vtiutil.read_vti(os.path.join(REF, "data", name))
        images[name] = {"shape": list(a.shape), "sha256": hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest(),
                        "porosity": float(1 - a.mean())}
    out = {
        "source": "jerome-lux/NS3D tests/results, README.md, tests/*.ini, data/*.vti",
        "test_spheres_ini": ini(os.path.join(REF, "tests/test_spheres.ini")),
        "compare_algorithms_ini": ini(os.path.join(REF, "tests/compare_algorithms.ini")),
        "res_header": header,
        "res_rows": rows,
        "info_head": info[:16],
        "info_counts": counts,
        "info_porosity_line": porosity_line,
        "info_initial_K": initial_k,
        "info_K_per_iteration": k_lines,
        "info_solve_lines": solves,
        "readme_64_table": table,
        "images": images,
    }
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_runs.json"))


if __name__ == "__main__":
    main()
