"""Benchmark of the NS3D permeability solve on GB300.

Workload (one GPU): a seeded 128^3 non-overlapping sphere pack (radius 8
voxels, porosity ~0.5, random sequential addition, seed 1), flow along x with
a unit pressure drop, mu = 1e-3, rho = 1, alpha = 0.5, BiCGSTAB tolerances
1e-8, outer convergence at RMR < 1e-6, plain FP64.  A step is one complete
permeability solve; steps cycle through SIMPLEC, SIMPLER (N1=2), SIMPLERR
(N1=2) and IDEAL (N1=N2=2).  Metric: permeability solves per second.

  value  solves/s with the image and geometry resident in HBM (each step
         resets the fields on the device and solves)
  e2e    solves/s through the C-ABI with host buffers: every step uploads the
         raw voxel image, builds the geometry, solves and downloads the fields
  roofline  the BiCGSTAB loop kernel (one persistent cooperative launch runs
         the iterations of a solve: K1 p/y, K2 v = A y + <r0,v>, K3 s/z,
         K4 t = A z + <t,t>,<t,s>, K5 x/r + <r0,r>,<r,r>) of the
         pressure(-correction) solves: algorithmic bytes per row-iteration
         (408 B by the fixed (45s+48) formula; the fused phases touch 360 B)
         over the kernel's CUDA-event time
  merged  a multi-image sample (8 device-generated images, edges 32-48,
         SIMPLEC capped at 150 outer iterations): one at a time, concurrent
         streams, merged solve sets and lockstep solves, FP64 and multilevel
         mixed precision, with the loop-grid autotuner's table
  readme_64  the reference's published benchmark case (its README's 64^3
         four-method table) solved here, beside the published CPU times
  cpu_baseline  the CPU oracle (the repo's restatement of the reference solver)
         on the first outer iterations of the same solve with every host core,
         scaled to a full solve by BiCGSTAB row-iterations

Multi-GPU: solves do not shard, so N GPUs run N independent replicas
(weak scaling); value = all ranks' solves / max elapsed over ranks.

`--impl reference` times the CPU oracle alone (the reference's own solver
cannot be built here: Eigen, Blitz++ and VTK are absent).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METHODS = ["SIMPLEC", "SIMPLER", "SIMPLERR", "IDEAL"]
SHAPE = (128, 128, 128)
RADIUS, TARGET_PHI, SEED = 8, 0.5, 1
# algorithmic bytes of one FP64 BiCGSTAB iteration per row, by the fixed
# formula (45s + 48) with s = 8: two SpMVs of (9s + 24) (7 coefficients, 6
# indices, x in, y out), two Jacobi applications of 3s, 21s of vector
# traffic.  The fused phases of the loop kernel touch 360 B (K1 48, K2 104,
# K3 40, K4 104, K5 64: the Jacobi products ride in the p and s updates).
LOOP_BYTES_PER_ROW = 408
LOOP_FUSED_BYTES_PER_ROW = 360
# FP64 instructions per row-iteration (a full 7-point row): two SpMVs (7 fma
# each), five dot-product fma, vector updates p 2, y 1, s 1, z 1, x 2, r 1
LOOP_FP64_PER_ROW = 27
# FP64 FMA throughput of this GPU, measured with a dependent-chain-free FMA
# loop over every SM (the tensor-core FP64 rate of GB300 is not used here)
FP64_PEAK_TFLOPS = 1.2

# BiCGSTAB row-iterations of one complete solve of this workload per method,
# measured by this benchmark's GPU arm; the CPU oracle follows the same
# trajectory bit for bit, so these scale its sampled cost to a full solve.
FULL_SOLVE_KRYLOV_ROWS = {"SIMPLEC": 246125574149, "SIMPLER": 316246186905, "SIMPLERR": 325991783660,
                          "IDEAL": 87945733905}
MAX_OUTER = 2000
PRECISION = 0  # 0 plain FP64, 1 mixed (FP32 inner / FP64 outer)


def workload_params(capi, lib, method):
    dx = 1e-6
    return capi.default_params(lib, dx=dx, dy=-1.0, dz=-1.0, mu=1e-3, rho=1.0, p0=1.0, gradp=1.0 / (SHAPE[0] * dx),
                               alpha=0.5, beta=1.0, vsolvertol=1e-8, psolvertol=1e-8, pcsolvertol=1e-8,
                               simpletol=1e-6, maxitsolver=2000, maxitSIMPLE=MAX_OUTER, N1=2, N2=2, porevalue=0,
                               direction=1, border=0, method=method, precision=PRECISION)


def make_image():
    from ns3d_gb300 import synth
    img, info = synth.rsa_spheres(SHAPE, RADIUS, TARGET_PHI, SEED)
    return img, info


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per row-iteration of the loop kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "krylov_loop_fp64_128.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_row_iteration:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_sample(capi, img, method, outer):
    """Oracle (CPU, all cores) on the first `outer` outer iterations."""
    from ns3d_gb300 import synth
    olib = os.path.join(ROOT, "oracle", "_build", "libns3d_oracle.so")
    if not os.path.exists(olib):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    lib = capi.load(olib)
    p = workload_params(capi, lib, method)
    p.maxitSIMPLE = outer
    s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
    t = time.perf_counter()
    r = s.solve()
    dt = time.perf_counter() - t
    s.close()
    return dt, r.krylov_rows, r


# Serving sample: a seeded stream of mixed permeability requests -- edges
# log-uniform in SERVE_EDGE (the serving mix spans 48-192; bounded here so a
# request takes seconds, not minutes), a sphere pack (radius 3-8, porosity
# 0.35-0.9) or a fibre pack (radius 2-4, porosity 0.7-0.95) generated on the
# device, flow along x, y or z, SIMPLEC or IDEAL.  Throughput is counted in
# equal windows of SERVE_WINDOW seconds: the plain FP64 path solves the stream
# one request at a time; the server (mixed precision, up to SERVE_ACTIVE in
# flight) receives Poisson arrivals at each rate of SERVE_RATES (a light load
# for latency, a saturating one for capacity); requests still queued when the
# window closes are dropped, those completed inside it are counted.  The
# first SERVE_PREPARED requests of the stream are generated before the
# windows start.
SERVE_EDGE = (32, 48)
SERVE_WINDOW = 30.0
SERVE_PREPARED = 200  # requests generated before the windows
SERVE_RATES = (1.0, 20.0)
SERVE_ACTIVE = 8
SERVE_PRECISION = 2  # mixed precision with the multilevel pressure preconditioner


def serving_request(capi, lib, i, seed=4):
    rng = np.random.default_rng([seed, i])
    shape = tuple(int(round(np.exp(rng.uniform(np.log(SERVE_EDGE[0]), np.log(SERVE_EDGE[1]))))) for _ in range(3))
    if rng.integers(2) == 0:
        kind, radius, phi = 0, int(rng.integers(3, 9)), float(rng.uniform(0.35, 0.9))
    else:
        kind, radius, phi = 1, int(rng.integers(2, 5)), float(rng.uniform(0.7, 0.95))
    img, ach, _ = capi.generate_image(lib, kind, shape, radius, phi, seed * 1000003 + i)
    return {"shape": shape, "raw": np.ascontiguousarray(img.transpose(2, 1, 0)).reshape(-1), "phi": ach,
            "kind": "spheres" if kind == 0 else "fibres", "direction": int(rng.integers(1, 4)),
            "method": [0, 3][int(rng.integers(2))]}


def request_params(capi, lib, r, precision):
    dx = 1e-6
    ext = r["shape"][r["direction"] - 1]
    return capi.default_params(lib, dx=dx, dy=-1.0, dz=-1.0, mu=1e-3, rho=1.0, p0=1.0, gradp=1.0 / (ext * dx),
                               alpha=0.5, beta=1.0, vsolvertol=1e-8, psolvertol=1e-8, pcsolvertol=1e-8,
                               simpletol=1e-6, maxitsolver=2000, maxitSIMPLE=MAX_OUTER, N1=2, N2=2, porevalue=0,
                               direction=r["direction"], border=0, method=r["method"], precision=precision)


def run_serving(capi, lib):
    """Windowed throughput: plain FP64 one request at a time vs the
    continuous-batching server in mixed precision under Poisson arrivals."""
    stream = [serving_request(capi, lib, i) for i in range(SERVE_PREPARED)]

    def req(i):
        return stream[i]

    k64 = {}
    t0 = time.perf_counter()
    n_plain = 0
    while time.perf_counter() - t0 < SERVE_WINDOW and n_plain < SERVE_PREPARED:
        r = req(n_plain)
        s = capi.Solver(lib, request_params(capi, lib, r, 0), r["raw"], r["shape"])
        k64[n_plain] = s.solve().K
        s.close()
        n_plain += 1
    plain_s = time.perf_counter() - t0
    out = {"workload": "seeded request stream: edges log-uniform %d-%d, sphere (r 3-8, phi 0.35-0.9) or fibre "
                       "(r 2-4, phi 0.7-0.95) packs generated on the device, flow x/y/z, SIMPLEC or IDEAL; "
                       "windows of %.0f s" % (SERVE_EDGE[0], SERVE_EDGE[1], SERVE_WINDOW),
           "plain_fp64_one_at_a_time": {"solves_per_s": n_plain / plain_s, "completed": n_plain,
                                        "seconds": plain_s}}
    for rate in SERVE_RATES:
        rng = np.random.default_rng(int(rate * 1000))
        srv = capi.Server(lib, SERVE_ACTIVE)
        subs = []
        t0 = time.perf_counter()
        nxt, j = 0.0, 0
        while True:
            now = time.perf_counter() - t0
            if now >= SERVE_WINDOW:
                break
            if j >= SERVE_PREPARED:  # every prepared request submitted: serve until the window closes
                time.sleep(max(0.0, SERVE_WINDOW - now))
                break
            if now >= nxt:
                r = req(j)
                ts = time.perf_counter() - t0
                subs.append((j, srv.submit(request_params(capi, lib, r, SERVE_PRECISION), r["raw"], r["shape"]), ts))
                j += 1
                nxt += rng.exponential(1.0 / rate)
            else:
                time.sleep(min(nxt - now, SERVE_WINDOW - now))
        cancelled = srv.cancel_queued()
        done, failed = [], 0
        for i, t, ts in subs:
            try:
                res, lat = srv.wait(t)
            except capi.NS3DError:
                failed += 1  # cancelled while queued, or failed
                continue
            done.append((i, ts + lat, lat, res.K))
        failed -= cancelled
        srv.stop()
        inside = sorted((d for d in done if d[1] <= SERVE_WINDOW), key=lambda d: d[1])
        lats = [d[2] for d in inside]
        # completion rate once the first request is through (the window count
        # also includes the initial ramp of a saturated server)
        steady = (len(inside) - 1) / (inside[-1][1] - inside[0][1]) if len(inside) > 2 else None
        errs = [abs(d[3] - k64[d[0]]) / abs(k64[d[0]]) for d in done if d[0] in k64]
        out["served_%s_rate_%g" % ("mixed_mg" if SERVE_PRECISION == 2 else "mixed", rate)] = {
            "arrival_rate_per_s": rate, "submitted": len(subs), "completed_in_window": len(inside),
            "failed": failed, "cancelled_in_queue": cancelled,
            "solves_per_s": len(inside) / SERVE_WINDOW,
            "steady_solves_per_s": steady,
            "steady_speedup_vs_plain_fp64": None if steady is None else steady / (n_plain / plain_s),
            "p50_latency_s": float(np.percentile(lats, 50)) if lats else None,
            "p99_latency_s": float(np.percentile(lats, 99)) if lats else None,
            "speedup_vs_plain_fp64": (len(inside) / SERVE_WINDOW) / (n_plain / plain_s),
            "K_compared": len(errs), "max_K_rel_err_vs_fp64": max(errs) if errs else None}
    out["max_active"] = SERVE_ACTIVE
    return out


# Batch sample (opt-in, --batch): a mix of uneven images -- each edge drawn from
# BATCH_EDGES per axis, a sphere pack (radius 3-8, porosity 0.35-0.9, overlap
# allowed) or a fibre pack (radius 2-4, porosity 0.7-0.95), generated on the
# device (ns3d_generate_image), flow along x, SIMPLEC -- solved by
# ns3d_batch_solve in mixed precision and, as the reference point, by the
# plain FP64 path one image at a time.
BATCH_IMAGES = 16
BATCH_EDGES = (32, 48, 64)


def run_batch(capi, lib, n_images, edges, max_concurrent):
    import ctypes as C
    rng = np.random.default_rng(3)
    imgs = []
    for i in range(n_images):
        shape = tuple(int(rng.choice(edges)) for _ in range(3))
        if rng.integers(2) == 0:
            kind, radius, phi = 0, int(rng.integers(3, 9)), float(rng.uniform(0.35, 0.9))
        else:
            kind, radius, phi = 1, int(rng.integers(2, 5)), float(rng.uniform(0.7, 0.95))
        img, ach, _ = capi.generate_image(lib, kind, shape, radius, phi, 1000 + i)
        imgs.append({"shape": shape, "raw": np.ascontiguousarray(img.transpose(2, 1, 0)).reshape(-1),
                     "kind": kind, "phi": ach, "direction": 1, "method": 0})
    k64, t64, cells = [], 0.0, 0
    for r in imgs:
        s = capi.Solver(lib, request_params(capi, lib, r, 0), r["raw"], r["shape"])
        t = time.perf_counter()
        res = s.solve()
        t64 += time.perf_counter() - t
        k64.append(res.K)
        cells += s.sizes.np * (res.iterations + 1)
        s.close()
    lib = capi._declare_server(lib)
    prm = (capi.Params * n_images)(*[request_params(capi, lib, r, SERVE_PRECISION) for r in imgs])
    ptrs = (C.POINTER(C.c_uint8) * n_images)(*[r["raw"].ctypes.data_as(C.POINTER(C.c_uint8)) for r in imgs])
    dims = np.array([d for r in imgs for d in r["shape"]], np.int32)
    res = (capi.Result * n_images)()
    status = np.zeros(n_images, np.int32)
    t = time.perf_counter()
    rc = lib.ns3d_batch_solve(prm, ptrs, dims.ctypes.data_as(C.POINTER(C.c_int32)), n_images, max_concurrent, res,
                              status.ctypes.data_as(C.POINTER(C.c_int32)))
    tb = time.perf_counter() - t
    rel = [abs(r.K - k) / abs(k) for r, k in zip(res, k64)]
    return {"workload": "%d images, edges from %s per axis, sphere (r 3-8, phi 0.35-0.9, overlapping) or fibre "
                        "(r 2-4, phi 0.7-0.95) packs generated on the device, SIMPLEC, flow x" % (n_images, edges),
            "status": int(rc),
            "plain_fp64_one_at_a_time": {"solves_per_s": n_images / t64, "seconds": t64,
                                         "cell_updates_per_s": cells / t64},
            "batch_mixed": {"solves_per_s": n_images / tb, "seconds": tb, "max_concurrent": max_concurrent,
                            "speedup_vs_plain_fp64": t64 / tb, "max_K_rel_err_vs_fp64": max(rel),
                            "K_rel_err_vs_fp64": rel}}


# Merged sample (in the default run, bounded; --no-merged skips it): the
# batch mix above with edges from MERGED_EDGES (SIMPLEC, flow x), solved in
# plain FP64 one image at a time, then as batches of concurrent solves on
# their own streams (ns3d_batch_solve), with their BiCGSTAB sets merged into
# shared persistent launches (ns3d_batch_solve_merged), and all driven in
# lockstep by one host thread (ns3d_batch_solve_lockstep), in plain FP64 and
# in the serving precision.  The FP64 legs follow the same trajectory bit for
# bit (fixed-order reductions), so MERGED_OUTER caps the outer iterations of
# every leg alike (the sample takes about half a minute).
MERGED_IMAGES = 8
MERGED_EDGES = (32, 48)
MERGED_OUTER = 150
MERGED_LANES = (1,)  # lanes of the solve group (cohorts of ceil(solves / lanes))


def run_merged(capi, lib, n_images, edges, max_concurrent, max_outer=2000):
    rng = np.random.default_rng(3)
    imgs = []
    for i in range(n_images):
        shape = tuple(int(rng.choice(edges)) for _ in range(3))
        if rng.integers(2) == 0:
            kind, radius, phi = 0, int(rng.integers(3, 9)), float(rng.uniform(0.35, 0.9))
        else:
            kind, radius, phi = 1, int(rng.integers(2, 5)), float(rng.uniform(0.7, 0.95))
        img, ach, _ = capi.generate_image(lib, kind, shape, radius, phi, 1000 + i)
        imgs.append({"shape": shape, "raw": np.ascontiguousarray(img.transpose(2, 1, 0)).reshape(-1),
                     "kind": kind, "phi": ach, "direction": 1, "method": 0})

    def prm(r, precision=0):
        p = request_params(capi, lib, r, precision)
        p.maxitSIMPLE = max_outer
        return p

    k1, t1, cells, rows = [], 0.0, 0, 0
    for r in imgs:
        s = capi.Solver(lib, prm(r), r["raw"], r["shape"])
        t = time.perf_counter()
        res = s.solve()
        t1 += time.perf_counter() - t
        k1.append(res.K)
        cells += s.sizes.np * (res.iterations + 1)
        rows += res.krylov_rows
        s.close()
    legs = {"plain_fp64_one_at_a_time": {"solves_per_s": n_images / t1, "seconds": t1,
                                         "cell_updates_per_s": cells / t1,
                                         "bicgstab_row_iterations_per_s": rows / t1}}
    mixed = "mixed_mg" if SERVE_PRECISION == 2 else "mixed"
    legs_spec = []
    for precision, label in ((0, "fp64"), (SERVE_PRECISION, mixed)):
        legs_spec.append(("batch_%s_streams" % label, 0, precision))
        for lanes in MERGED_LANES:
            legs_spec.append(("batch_%s_merged_%d_lane%s" % (label, lanes, "s" if lanes > 1 else ""), lanes,
                              precision))
        legs_spec.append(("batch_%s_lockstep" % label, -1, precision))
    for name, merged, precision in legs_spec:
        t = time.perf_counter()
        if merged >= 0:
            res, status, g, rc = capi.batch_solve(lib, [prm(r, precision) for r in imgs], [r["raw"] for r in imgs],
                                                  [r["shape"] for r in imgs], max_concurrent, merged=merged)
        else:  # every image resident, all driven in lockstep by one thread
            res, status, rc = capi.batch_solve_lockstep(lib, [prm(r, precision) for r in imgs],
                                                        [r["raw"] for r in imgs], [r["shape"] for r in imgs])
            g = None
        dt = time.perf_counter() - t
        leg = {"solves_per_s": n_images / dt, "seconds": dt, "status": int(rc),
               "speedup_vs_one_at_a_time": t1 / dt, "max_concurrent": max_concurrent}
        if precision == 0:
            leg.update({"cell_updates_per_s": cells / dt, "bicgstab_row_iterations_per_s": rows / dt,
                        "K_bit_identical_to_one_at_a_time": all(x.K == k for x, k in zip(res, k1))})
        else:
            leg["max_K_rel_err_vs_fp64"] = max(abs(x.K - k) / abs(k) for x, k in zip(res, k1))
            leg["outer_iterations"] = [int(x.iterations) for x in res]
        if g is not None:
            leg["lanes"] = merged
            leg["group"] = g.as_dict()
            leg["mean_systems_per_set"] = g.systems / max(g.launches, 1)
        legs[name] = leg
    legs["autotune_table"] = capi.autotune_table(lib).splitlines()
    legs["workload"] = ("%d images, edges from %s per axis, sphere (r 3-8, phi 0.35-0.9, overlapping) or fibre "
                        "(r 2-4, phi 0.7-0.95) packs generated on the device, SIMPLEC, flow x, plain FP64, "
                        "at most %d outer iterations" % (n_images, edges, max_outer))
    return legs


# The reference's own published benchmark (README.md:181-187 of
# jerome-lux/NS3D): tests/compare_algorithms.ini on data/spheres_64.vti (a
# regular 64^3 sphere lattice, regenerated here byte for byte), the four
# methods, wall times on an unstated CPU with 4 OpenMP threads.  Each method
# is solved here in plain FP64 (image upload, geometry build and solve
# timed together; the reference's times also include reading the file).
README_64 = {"SIMPLEC": (3.28386e-12, 48, 5.435), "SIMPLER": (3.28382e-12, 42, 8.033),
             "SIMPLERR": (3.28175e-12, 23, 5.690), "IDEAL": (3.28212e-12, 19, 2.788)}


def readme64_params(capi, lib, method):
    return capi.default_params(lib, dx=2e-6, dy=-1.0, dz=-1.0, mu=1e-3, rho=1e3, p0=1e5, gradp=1e2, alpha=0.8,
                               beta=1.0, vsolvertol=1e-5, psolvertol=1e-6, pcsolvertol=1e-3, simpletol=1e-4,
                               deltaRMR=1e-4, maxitsolver=500, maxitSIMPLE=200, N1=2, N2=2, porevalue=0,
                               direction=1, border=0, method=method, precision=0)


def run_readme64(capi, lib):
    from ns3d_gb300 import synth
    img = synth.sphere_lattice(64, 8, 3)
    raw = synth.to_raw(img)
    out = {"case": "README 64^3 compare_algorithms table (sphere lattice, 4 methods), plain FP64",
           "published_hardware": "CPU, 4 OpenMP threads (model unstated)"}
    warm = readme64_params(capi, lib, "SIMPLEC")  # untimed: device context and module loading
    warm.maxitSIMPLE = 1
    capi.Solver(lib, warm, raw, img.shape).close()
    for m, (k_pub, it_pub, sec_pub) in README_64.items():
        t = time.perf_counter()
        s = capi.Solver(lib, readme64_params(capi, lib, m), raw, img.shape)
        r = s.solve()
        dt = time.perf_counter() - t
        s.close()
        out[m] = {"seconds": dt, "K": r.K, "outer_iterations": int(r.iterations), "converged": int(r.converged),
                  "published_seconds": sec_pub, "published_K": k_pub, "published_iterations": it_pub,
                  "K_rel_diff_vs_published": abs(r.K - k_pub) / k_pub, "speedup_vs_published": sec_pub / dt}
    return out


# Large sample (opt-in, --large): a 256^3 image of isotropic
# straight fibres of radius 3, porosity ~0.85, seed 2, flow along z --
# generated on the device; the first LARGE_OUTER outer SIMPLEC iterations in
# plain FP64 and in mixed precision: time per outer iteration and the
# FP32/FP64 time ratio (a converged 256^3 solve takes many minutes).
LARGE_OUTER = 10


def run_large(capi, lib, outer):
    img, ach, _ = capi.generate_image(lib, 1, (256, 256, 256), 3, 0.85, 2)
    raw = np.ascontiguousarray(img.transpose(2, 1, 0)).reshape(-1)
    r = {"shape": (256, 256, 256), "direction": 3, "method": 0}
    out = {"workload": "256^3 fibres r=3 phi=%.4f seed 2 (device generator), flow z, SIMPLEC, first %d outer "
                       "iterations" % (ach, outer)}
    for prec, name in ((0, "fp64"), (1, "mixed"), (2, "mixed_mg")):
        p = request_params(capi, lib, r, prec)
        p.maxitSIMPLE = outer
        s = capi.Solver(lib, p, raw, img.shape)
        t = time.perf_counter()
        res = s.solve()
        dt = time.perf_counter() - t
        out[name] = {"seconds": dt, "seconds_per_outer_iteration": dt / max(res.iterations, 1),
                     "outer_iterations": res.iterations, "K": res.K, "krylov_iterations": res.krylov_iterations,
                     "np": s.sizes.np}
        s.close()
    out["fp32_fp64_time_ratio"] = out["mixed"]["seconds"] / out["fp64"]["seconds"]
    out["mixed_mg_fp64_time_ratio"] = out["mixed_mg"]["seconds"] / out["fp64"]["seconds"]
    out["K_rel_diff_at_this_iteration"] = abs(out["mixed"]["K"] - out["fp64"]["K"]) / abs(out["fp64"]["K"])
    out["K_rel_diff_mg_at_this_iteration"] = abs(out["mixed_mg"]["K"] - out["fp64"]["K"]) / abs(out["fp64"]["K"])
    return out


def run_reference(args):
    from ns3d_gb300 import capi
    world, rank, _, dist = dist_setup()
    if rank != 0:
        return 0
    img, info = make_image()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    outer = 2
    rates = []
    for i in range(args.warmup + args.steps):
        m = METHODS[i % len(METHODS)]
        dt, rows, _ = cpu_sample(capi, img, m, outer)
        full = FULL_SOLVE_KRYLOV_ROWS.get(m)
        if i >= args.warmup:
            rates.append((dt, rows, full))
    tot_time = sum(dt * (full / rows if full else 1.0) for dt, rows, full in rates)
    value = len(rates) / tot_time
    line = {"impl": "reference", "metric": "permeability solves/s (128^3 sphere pack, 4 SIMPLE-family methods)",
            "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot_time / len(rates), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "128^3 RSA spheres r=8 phi~%.3f seed 1, SIMPLEC/SIMPLER/SIMPLERR/IDEAL" %
                       info["porosity"], "global_batch": 1, "parallelism": "replicas"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port",
                             "sample": "first %d outer iterations of each step's solve, scaled to a full solve "
                                       "by BiCGSTAB row-iterations" % outer},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    global PRECISION
    import ns3d_gb300
    from ns3d_gb300 import capi, synth
    world, rank, local, dist = dist_setup()
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local)) if world > 1 else None
    lib = ns3d_gb300.lib()
    img, info = make_image()
    raw = synth.to_raw(img)
    solvers = {}
    for m in METHODS:
        s = capi.Solver(lib, workload_params(capi, lib, m), raw, img.shape)
        solvers[m] = s
    sizes = solvers[METHODS[0]].sizes

    def step(i):
        s = solvers[METHODS[i % len(METHODS)]]
        s.set_initial_fields()
        return s.solve()

    for i in range(args.warmup):
        step(i)
    for s in solvers.values():
        s.set_profiling(True)
    clocks = Clocks(local) if rank == 0 else None
    barrier(dist)
    t0 = time.perf_counter()
    results = [step(i) for i in range(args.steps)]
    elapsed = time.perf_counter() - t0
    clk = clocks.stop() if clocks else None
    barrier(dist)
    elapsed = reduce_max(dist, elapsed)
    value = world * args.steps / elapsed
    # per-kernel profile of the pressure(-correction) BiCGSTAB
    tot = {"ms": [0.0] * 6, "launches": [0] * 6, "rows": [0] * 6}
    gpu_launches = int(solvers[METHODS[0]].profile().total_launches)
    for s in solvers.values():
        p = s.profile()
        for k in range(6):
            tot["ms"][k] += p.ms[k]
            tot["launches"][k] += p.launches[k]
            tot["rows"][k] += p.rows[k]
        s.set_profiling(False)
    loop_ms, loop_launches, loop_rows = tot["ms"][5], tot["launches"][5], tot["rows"][5]
    peak, peak_kind = load_peaks()
    achieved = LOOP_BYTES_PER_ROW * loop_rows / (loop_ms * 1e-3) / 1e9 if loop_ms > 0 else 0.0
    fp64_tflops = LOOP_FP64_PER_ROW * loop_rows / (loop_ms * 1e-3) / 1e12 if loop_ms > 0 else 0.0
    traffic = ncu_traffic()
    kr_rows = {METHODS[i % len(METHODS)]: int(results[i].krylov_rows) for i in range(len(results))}
    outer_its = {METHODS[i % len(METHODS)]: int(results[i].iterations) for i in range(len(results))}
    ks = {METHODS[i % len(METHODS)]: float(results[i].K) for i in range(len(results))}
    cell_updates = sum(sizes.np * (r.iterations + 1) for r in results)
    # end to end through the C-ABI with host buffers
    e2e_steps = 0 if args.no_e2e else min(args.steps, 2)
    h2d = raw.nbytes
    d2h = 8 * (sizes.np + sizes.nu + sizes.nv + sizes.nw)
    barrier(dist)
    t1 = time.perf_counter()
    for i in range(e2e_steps):
        m = METHODS[i % len(METHODS)]
        s = capi.Solver(lib, workload_params(capi, lib, m), raw, img.shape)
        s.solve()
        f = s.fields()
        s.close()
        assert f[0].size == sizes.np
    e2e_elapsed = reduce_max(dist, time.perf_counter() - t1)
    e2e_value = world * e2e_steps / e2e_elapsed if e2e_steps else None
    # the same workload in mixed precision with the multilevel pressure
    # preconditioner: one solve per method, K against that method's FP64 solve
    mixed_mg = None
    if args.mixed_mg and world == 1:
        saved, PRECISION = PRECISION, 2
        t_mg, errs, its = 0.0, {}, {}
        for m in METHODS:
            s = capi.Solver(lib, workload_params(capi, lib, m), raw, img.shape)
            t = time.perf_counter()
            res = s.solve()
            t_mg += time.perf_counter() - t
            s.close()
            its[m] = int(res.iterations)
            if m in ks:
                errs[m] = abs(res.K - ks[m]) / abs(ks[m])
        PRECISION = saved
        mixed_mg = {"solves_per_s": len(METHODS) / t_mg, "seconds_per_solve": t_mg / len(METHODS),
                    "speedup_vs_plain_fp64": (len(METHODS) / t_mg) / value, "outer_iterations": its,
                    "K_rel_err_vs_fp64": errs}
    serving = None
    if args.serving and world == 1:
        serving = run_serving(capi, lib)
    large = run_large(capi, lib, args.large_outer) if (args.large and world == 1) else None
    batch = None
    if args.batch and world == 1:
        batch = run_batch(capi, lib, args.batch_images, tuple(int(x) for x in args.batch_edges.split(",")),
                          SERVE_ACTIVE)
    readme64 = None
    if args.readme64 and world == 1:
        try:
            readme64 = run_readme64(capi, lib)
        except Exception as e:  # a failed sample is reported, the bench line still printed
            readme64 = {"error": repr(e)}
    merged = None
    if args.merged and world == 1:
        try:
            merged = run_merged(capi, lib, args.merged_images, tuple(int(x) for x in args.merged_edges.split(",")),
                                SERVE_ACTIVE, max_outer=args.merged_outer)
        except Exception as e:  # a failed sample is reported, the bench line still printed
            merged = {"error": repr(e)}
    line = None
    if rank == 0:
        cpu = None
        if args.cpu_baseline and world == 1:
            dt, rows, _ = cpu_sample(capi, img, "SIMPLEC", 2)
            full = kr_rows.get("SIMPLEC")
            cpu_time = dt * full / rows
            cpu = {"value": 1.0 / cpu_time, "unit": "solves/s", "cores": int(os.environ.get("OMP_NUM_THREADS",
                                                                                             os.cpu_count())),
                   "kind": "port",
                   "sample": "CPU oracle, first 2 outer SIMPLEC iterations of the same 128^3 solve (%.1f s), "
                             "scaled by BiCGSTAB row-iterations to the full solve" % dt}
        line = {"metric": "permeability solves/s (128^3 sphere pack, 4 SIMPLE-family methods)",
                "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "128^3 RSA spheres r=8 phi=%.4f seed 1, SIMPLEC/SIMPLER/SIMPLERR/IDEAL "
                                       "cycled per step" % info["porosity"],
                           "global_batch": world, "seq_len": None, "parallelism": "replicas x%d" % world,
                           "np": sizes.np, "nu": sizes.nu, "nv": sizes.nv, "nw": sizes.nw,
                           "l2": "working set (matrices + Krylov vectors) > 129 MB L2; no flush",
                           "outer_iterations": outer_its, "K": ks,
                           "cell_updates_per_s": cell_updates / elapsed * world},
                "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "roofline": {"bound": "hbm", "kernel": "k_kr_loop (BiCGSTAB iterations of the pressure solves)",
                             "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                             "peak_kind": peak_kind,
                             "traffic": None if traffic is None else traffic * loop_rows / max(loop_launches, 1),
                             "traffic_bytes_per_row_iteration": traffic,
                             "bytes_per_row_iteration": LOOP_BYTES_PER_ROW,
                             "fused_bytes_per_row_iteration": LOOP_FUSED_BYTES_PER_ROW,
                             "achieved_fused_bytes": achieved * LOOP_FUSED_BYTES_PER_ROW / LOOP_BYTES_PER_ROW,
                             "fp64_tflops": fp64_tflops, "fp64_peak_tflops": FP64_PEAK_TFLOPS,
                             "fp64_frac": fp64_tflops / FP64_PEAK_TFLOPS,
                             "avg_launch_ms": loop_ms / max(loop_launches, 1),
                             "row_iterations_per_launch": loop_rows / max(loop_launches, 1)},
                "kernels": dict({n: {"iterations": tot["launches"][k], "ms": round(tot["ms"][k], 3)}
                                 for k, n in enumerate(["K1_p", "K2_spmv_v", "K3_s", "K4_spmv_t", "K5_xr"])},
                                k_kr_loop={"launches": loop_launches, "ms": round(loop_ms, 3)}),
                "gpu_launches": gpu_launches,
                "krylov_rows": kr_rows,
                "cpu_baseline": cpu,
                "mixed_mg": mixed_mg,
                "serving": serving,
                "batch": batch,
                "merged": merged,
                "readme_64": readme64,
                "large": large,
                "clocks": clk}
        print(json.dumps(line))
    for s in solvers.values():
        s.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    global METHODS, MAX_OUTER, PRECISION, SERVE_WINDOW, SERVE_EDGE, SERVE_ACTIVE, SERVE_PRECISION, MERGED_LANES
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-serving", dest="serving", action="store_false",
                    help="skip the serving sample (plain FP64 one at a time vs the mixed-precision server)")
    ap.add_argument("--serving-window", type=float, default=SERVE_WINDOW, help="seconds per throughput window")
    ap.add_argument("--serving-edge", default="%d,%d" % SERVE_EDGE, help="min,max image edge of the requests")
    ap.add_argument("--serving-active", type=int, default=SERVE_ACTIVE, help="solves in flight at most")
    ap.add_argument("--batch", action="store_true", help="add the batch sample (opt-in: a few minutes)")
    ap.add_argument("--large", action="store_true", help="add the 256^3 fibre-pack sample (opt-in)")
    ap.add_argument("--no-readme64", dest="readme64", action="store_false",
                    help="skip the reference's published 64^3 four-method case")
    ap.add_argument("--no-merged", dest="merged", action="store_false",
                    help="skip the multi-image sample (one at a time, streams, merged sets, lockstep)")
    ap.add_argument("--merged-images", type=int, default=MERGED_IMAGES)
    ap.add_argument("--merged-edges", default=",".join(str(e) for e in MERGED_EDGES))
    ap.add_argument("--merged-outer", type=int, default=MERGED_OUTER)
    ap.add_argument("--merged-lanes", default=",".join(str(x) for x in MERGED_LANES),
                    help="lane counts of the merged legs")
    ap.add_argument("--no-mixed-mg", dest="mixed_mg", action="store_false",
                    help="skip the workload's solves in mixed precision with the multilevel preconditioner")
    ap.add_argument("--large-outer", type=int, default=LARGE_OUTER)
    ap.add_argument("--batch-images", type=int, default=BATCH_IMAGES)
    ap.add_argument("--batch-edges", default=",".join(str(e) for e in BATCH_EDGES))
    ap.add_argument("--methods", default=",".join(METHODS), help="comma-separated subset of the four methods")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "mixed_mg"])
    ap.add_argument("--serving-precision", default="mixed_mg", choices=["mixed", "mixed_mg"],
                    help="precision of the served solves")
    ap.add_argument("--max-outer", type=int, default=2000,
                    help="cap on outer iterations (maxitSIMPLE); below 2000 only for short profiling runs")
    args = ap.parse_args()
    MERGED_LANES = tuple(int(x) for x in args.merged_lanes.split(",") if x.strip())
    SERVE_WINDOW = args.serving_window
    SERVE_EDGE = tuple(int(x) for x in args.serving_edge.split(","))
    SERVE_ACTIVE = args.serving_active
    METHODS = [m.strip().upper() for m in args.methods.split(",") if m.strip()]
    MAX_OUTER = args.max_outer
    PRECISION = {"fp64": 0, "mixed": 1, "mixed_mg": 2}[args.precision]
    SERVE_PRECISION = 1 if args.serving_precision == "mixed" else 2
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
