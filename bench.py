"""Benchmark of the NS3D permeability solve on GB300.

Metric: permeability solves/s and p50/p99 latency of the served solver at
|dK/K| <= 1e-4 against the plain FP64 GPU path.

Workload -- the serving stream (ns3d_gb300/workloads.py): a seeded Poisson
stream of permeability requests; request i is a cube image of edge
log-uniform in [48, 192] voxels, a pack of overlapping spheres (radius 3-8)
or of isotropic straight fibres (radius 2-4), porosity uniform in
[0.35, 0.95], rasterised on the device; flow along x, y or z; SIMPLEC or
IDEAL.  Creeping-flow physics (dx = 1e-6 m, mu = 1e-3, rho = 1, unit
pressure drop along the flow); the outer-loop settings of the reference's
own benchmark input (its tests/compare_algorithms.ini: alpha 0.8,
convergence at RMR < 1e-4) with BiCGSTAB tolerances 1e-8 (at most 2000
iterations), so that every served K can be held to 1e-4 of its plain FP64 K.

A step is one request: `--warmup W` requests are served untimed, then the
next `--steps K` requests are timed in every leg.

  plain_fp64  the K requests solved one at a time on the plain FP64 path
              (the reference's solver restated bit for bit), images already
              in HBM: the baseline the metric is quoted against
  value       the same K requests served by the continuous-batching server
              (mixed precision: FP32 inner solves with the multilevel
              pressure preconditioner inside FP64 defect correction; at most
              SERVE_ACTIVE solves in flight, admitted by free HBM), arriving
              as a Poisson stream at SAT_RATE requests/s (saturating: every
              request is queued within a second); images already in HBM
              (ns3d_server_submit_resident with device pointers), fields
              left on the device.  value = K / (first arrival -> last
              completion); p50/p99 latency (arrival -> completion) and the
              |dK/K| of every request against its plain FP64 solve
  e2e         the same K requests through the same C-ABI from pinned host
              images, every request's fields read back to host memory
  rate_sweep  throughput and p50/p99 latency at the arrival rates of
              SWEEP_RATES (SWEEP_REQUESTS further requests of the stream each)
  roofline    the FP64 BiCGSTAB loop kernel k_kr_loop of the plain FP64 leg
              (one persistent cooperative launch per pressure solve): 408 B
              per row-iteration by the fixed (45s+48) formula over its
              CUDA-event time, against MEASURED_PEAKS.json
  cpu_baseline  complete CPU-oracle solves of the 64^3 sphere pack
              (workloads.sphere64: radius 6, porosity 0.55, SIMPLEC,
              tolerances 1e-8, RMR < 1e-6) with every physical host core
              and with 4 threads (the reference README's thread count;
              --no-cpu-4-threads skips it), beside the plain FP64 GPU solve
              of the same case
  batch64     (opt-in, --batch64) 64 uneven images (edges from {32..96} per axis, sphere or fibre
              packs, SIMPLEC, flow x) solved one at a time in plain FP64 and
              together in mixed precision on concurrent streams, as merged
              persistent launches over the ragged chunk list, and in lockstep
              from one host thread: aggregate cell-updates/s and every
              image's |dK/K| against plain FP64
  readme_64   the reference's published 64^3 four-method table, solved here

The served legs' times are wall time between device synchronizations (their
work spans many streams); kernel-level figures come from CUDA events.

Multi-GPU: solves do not shard; N GPUs serve N independent streams (replicas,
weak scaling), value = all ranks' solves / max elapsed over ranks.

`--impl reference` is the reference arm: the reference's solver cannot be
built here (Eigen, Blitz++ and VTK are absent), so its CPU restatement (the
oracle) stands in for it, and a complete CPU solve of a stream request takes
minutes to hours -- the arm reports itself unavailable with that reason.
"""
import argparse
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

T_START = time.perf_counter()
METRIC = "permeability solves/sec and p50/p99 latency at |dK/K|<=1e-4 vs plain FP64 GPU"
MAX_OUTER = 2000
SAT_RATE = 20.0            # arrivals per second of the timed legs (saturating)
SWEEP_RATES = (0.5, 1.0, 2.0, 5.0, 10.0)
SWEEP_REQUESTS = 6         # requests per rate of the sweep
SERVE_ACTIVE = 8           # solves in flight at most
SERVE_PRECISION = 2        # mixed precision with the multilevel pressure preconditioner
K_TOL = 1e-4               # |dK/K| bar of the metric
# algorithmic bytes of one FP64 BiCGSTAB iteration per row, by the fixed
# formula (45s + 48) with s = 8: two SpMVs of (9s + 24) (7 coefficients, 6
# indices, x in, y out), two Jacobi applications of 3s, 21s of vector
# traffic.  The fused phases of the loop kernel touch 360 B (K1 48, K2 104,
# K3 40, K4 104, K5 64: the Jacobi products ride in the p and s updates).
LOOP_BYTES_PER_ROW = 408
LOOP_FUSED_BYTES_PER_ROW = 360


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



# parameters of the readme_64 and large samples
def request_params(capi, lib, r, precision):
    dx = 1e-6
    ext = r["shape"][r["direction"] - 1]
    return capi.default_params(lib, dx=dx, dy=-1.0, dz=-1.0, mu=1e-3, rho=1.0, p0=1.0, gradp=1.0 / (ext * dx),
                               alpha=0.5, beta=1.0, vsolvertol=1e-8, psolvertol=1e-8, pcsolvertol=1e-8,
                               simpletol=1e-6, maxitsolver=2000, maxitSIMPLE=MAX_OUTER, N1=2, N2=2, porevalue=0,
                               direction=r["direction"], border=0, method=r["method"], precision=precision)




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


def physical_cores():
    """Physical host cores (distinct core/socket pairs of lscpu -p)."""
    try:
        out = subprocess.run(["lscpu", "-p=CORE,SOCKET"], capture_output=True, text=True, check=True).stdout
        pairs = {l for l in out.splitlines() if l and not l.startswith("#")}
        if pairs:
            return len(pairs)
    except Exception:
        pass
    return os.cpu_count() or 1


# ---- the serving stream -----------------------------------------------------------
def materialize(capi, lib, req, torch, dev):
    """Generate a request's image on the device; keep it in HBM (for the
    resident legs) and in pinned host memory (for the end-to-end leg)."""
    img, ach, _ = capi.generate_image(lib, req["kind"], req["shape"], req["radius"], req["porosity"],
                                      req["image_seed"])
    raw = np.ascontiguousarray(img.transpose(2, 1, 0)).reshape(-1)
    host = torch.from_numpy(raw).pin_memory()
    d = host.to(dev)
    out = dict(req)
    out.update(achieved_porosity=ach, host=host, dev=d, nbytes=raw.nbytes)
    return out


def note(*a):
    """Progress on stderr (the JSON line is the only stdout output)."""
    print("[bench %.0f s]" % (time.perf_counter() - T_START), *a, file=sys.stderr, flush=True)


def describe(it):
    return {"edge": it["shape"][0], "pack": "spheres" if it["kind"] == 0 else "fibres", "radius": it["radius"],
            "porosity": round(it["achieved_porosity"], 4), "direction": "xyz"[it["direction"] - 1],
            "method": it["method"]}


def plain_leg(capi, workloads, lib, items, torch):
    """Every request solved alone on the plain FP64 path; the loop kernel's
    CUDA-event time and row-iterations of the pressure solves."""
    recs, prof = [], {"ms": 0.0, "launches": 0, "rows": 0, "phase_ms": [0.0] * 5, "iters": 0}
    total = 0.0
    for it in items:
        torch.cuda.synchronize()
        t = time.perf_counter()
        s = capi.Solver(lib, workloads.stream_params(capi, lib, it, 0), it["dev"].data_ptr(), it["shape"])
        s.set_profiling(True)
        r = s.solve()
        p = s.profile()
        sizes = (s.sizes.np, s.sizes.nu, s.sizes.nv, s.sizes.nw)
        s.close()
        dt = time.perf_counter() - t
        total += dt
        prof["ms"] += p.ms[5]
        prof["launches"] += p.launches[5]
        prof["rows"] += p.rows[5]
        prof["iters"] += p.launches[0]
        for k in range(5):
            prof["phase_ms"][k] += p.ms[k]
        recs.append({"seconds": dt, "K": r.K, "outer_iterations": int(r.iterations), "converged": int(r.converged),
                     "sizes": sizes})
    return total, recs, prof


def serve_leg(capi, workloads, lib, items, rate, seed, torch, resident=True, keep_fields=False, sizes=None):
    """Serve `items` under Poisson arrivals at `rate`/s: returns elapsed (first
    arrival -> last result in hand), per-request (K, latency, iterations),
    failures, the kernel launches of the region and the bytes read back."""
    srv = capi.Server(lib, SERVE_ACTIVE)
    gaps = np.random.default_rng(seed).exponential(1.0 / rate, len(items))
    arrive = np.concatenate([[0.0], np.cumsum(gaps[1:])])
    params = [workloads.stream_params(capi, lib, it, SERVE_PRECISION) for it in items]
    torch.cuda.synchronize()
    l0 = lib.ns3d_kernel_launches()
    t0 = time.perf_counter()
    tickets = []
    for k, it in enumerate(items):
        delay = t0 + arrive[k] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        ptr = it["dev"].data_ptr() if resident else it["host"].data_ptr()
        tickets.append(srv.submit_resident(params[k], ptr, it["shape"], keep_fields))
    out, failed, d2h = [], 0, 0
    for k, t in enumerate(tickets):
        try:
            r, lat = srv.wait(t)
        except capi.NS3DError:
            failed += 1
            out.append(None)
            continue
        if keep_fields:
            f = srv.fields(t, sizes[k])
            d2h += sum(a.nbytes for a in f)
        out.append({"K": r.K, "latency_s": lat, "outer_iterations": int(r.iterations), "converged": int(r.converged)})
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    launches = lib.ns3d_kernel_launches() - l0
    srv.stop()
    return elapsed, out, failed, launches, d2h


def latency_stats(recs):
    lats = [r["latency_s"] for r in recs if r]
    if not lats:
        return None, None
    return float(np.percentile(lats, 50)), float(np.percentile(lats, 99))


# ---- many images at once: the 64-image batch ------------------------------------------
def run_batch64(capi, workloads, lib, torch, dev, n_images):
    """The 64-image batch (workloads.batch64_request): plain FP64 one image at
    a time (the K reference), then the images solved together in mixed
    precision with the multilevel pressure preconditioner -- on concurrent
    streams (ns3d_batch_solve), with their BiCGSTAB sets merged into shared
    persistent launches over the ragged chunk list (ns3d_batch_solve_merged),
    and driven in lockstep by one host thread (ns3d_batch_solve_lockstep).
    Aggregate cell-updates/s (fluid pressure cells x outer iterations) and
    every image's |dK/K| against its plain FP64 solve."""
    items = [materialize(capi, lib, workloads.batch64_request(i), torch, dev) for i in range(n_images)]
    raws = [it["host"].numpy() for it in items]
    k64, nps, cells64, t64 = [], [], 0, 0.0
    for it in items:
        torch.cuda.synchronize()
        t = time.perf_counter()
        s = capi.Solver(lib, workloads.stream_params(capi, lib, it, 0), it["dev"].data_ptr(), it["shape"])
        r = s.solve()
        s.close()
        t64 += time.perf_counter() - t
        k64.append(r.K)
        nps.append(s.sizes.np)
        cells64 += s.sizes.np * (r.iterations + 1)
    out = {"workload": "%d images, each edge from {32,48,64,80,96}, sphere (r 3-8, phi 0.35-0.9) or fibre "
                       "(r 2-4, phi 0.7-0.95) packs generated on the device, SIMPLEC, flow x" % n_images,
           "plain_fp64_one_at_a_time": {"solves_per_s": n_images / t64, "seconds": t64,
                                        "cell_updates_per_s": cells64 / t64}}
    prm = [workloads.stream_params(capi, lib, it, SERVE_PRECISION) for it in items]
    dims = [it["shape"] for it in items]
    for name, merged in (("streams", 0), ("merged", 1), ("lockstep", -1)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        if merged >= 0:
            res, st, g, rc = capi.batch_solve(lib, prm, raws, dims, SERVE_ACTIVE, merged=merged)
        else:
            res, st, rc = capi.batch_solve_lockstep(lib, prm, raws, dims)
        dt = time.perf_counter() - t
        cells = sum(n * (r.iterations + 1) for n, r in zip(nps, res))
        errs = [abs(r.K - k) / abs(k) if k else None for r, k in zip(res, k64)]
        valid = [e for e in errs if e is not None]
        out["mixed_mg_" + name] = {"solves_per_s": n_images / dt, "seconds": dt, "status": int(rc),
                                   "cell_updates_per_s": cells / dt, "speedup_vs_plain_fp64": t64 / dt,
                                   "max_K_rel_err_vs_fp64": max(valid) if valid else None,
                                   "outer_iterations": [int(r.iterations) for r in res]}
    return out


# ---- CPU baseline: complete oracle solves --------------------------------------------
CPU_CHILD = r"""
import json, sys, time
sys.path.insert(0, %(root)r)
from ns3d_gb300 import capi, synth, workloads
lib = capi.load(%(lib)r)
img, info = workloads.sphere64()
p = workloads.solve_params(capi, lib, 64, "SIMPLEC", 1, 0)
s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
t = time.perf_counter()
r = s.solve()
dt = time.perf_counter() - t
rec = {"seconds": dt, "K": r.K, "outer_iterations": int(r.iterations), "converged": int(r.converged)}
import ctypes as C
ph = (C.c_double * 4)()
if hasattr(lib, "ns3d_oracle_phase_seconds") and lib.ns3d_oracle_phase_seconds(ph) == 0:
    rec["phase_seconds"] = {"assembly": ph[0], "bicgstab": ph[1], "corrections": ph[2], "diagnostics": ph[3],
                            "other": dt - sum(ph)}
print(json.dumps(rec))
"""


def oracle_complete_solve(threads):
    """One complete CPU-oracle solve of the 64^3 sphere pack with `threads`
    OpenMP threads (own process: the thread count is read when OpenMP starts)."""
    olib = os.path.join(ROOT, "oracle", "_build", "libns3d_oracle.so")
    if not os.path.exists(olib):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="close")
    p = subprocess.run([sys.executable, "-c", CPU_CHILD % {"root": ROOT, "lib": olib}], env=env,
                       capture_output=True, text=True, check=True)
    return json.loads(p.stdout.strip().splitlines()[-1])


def gpu_sphere64(capi, workloads, lib):
    """The plain FP64 GPU solve of the same 64^3 case (image from the host)."""
    from ns3d_gb300 import synth
    img, info = workloads.sphere64()
    raw = synth.to_raw(img)
    p = workloads.solve_params(capi, lib, 64, "SIMPLEC", 1, 0)
    capi.Solver(lib, p, raw, img.shape).close()  # untimed: first open
    t = time.perf_counter()
    s = capi.Solver(lib, p, raw, img.shape)
    r = s.solve()
    s.fields()
    s.close()
    return {"seconds": time.perf_counter() - t, "K": r.K, "outer_iterations": int(r.iterations),
            "porosity": info["porosity"]}


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
    """The reference arm: unavailable for this workload (see the docstring)."""
    world, rank, _, dist = dist_setup()
    if rank != 0:
        return 0
    rec = None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "oracle_sphere128_SIMPLEC.json")) as f:
            rec = json.load(f)["oracle"]
    except Exception:
        pass
    why = ("the reference's own solver cannot be built here (Eigen, Blitz++ and VTK are absent) and its CPU "
           "restatement needs minutes to hours per complete solve of a request of this stream (edges 48-192)")
    if rec:
        why += " (a converged 128^3 sphere-pack SIMPLEC solve took %.0f s on %d %s cores)" % (
            rec["seconds"], rec["threads"], rec.get("host", "host"))
    why += ", so %d complete solves do not fit one run; complete CPU solves of the 64^3 case are the GPU " \
           "line's cpu_baseline" % (args.warmup + args.steps)
    print(json.dumps({"impl": "reference", "metric": METRIC, "unavailable": why}))
    return 0


def run_gpu(args):
    import ns3d_gb300
    import torch
    from ns3d_gb300 import capi, workloads
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(0 if world == 1 else local)
    dev = torch.device("cuda", torch.cuda.current_device())
    lib = ns3d_gb300.lib()
    W, K = args.warmup, args.steps
    base = args.first + rank * 100000  # each replica serves its own part of the stream
    items = [materialize(capi, lib, workloads.stream_request(base + i), torch, dev) for i in range(W + K)]
    warm, timed = items[:W], items[W:]
    note("stream ready: edges", [it["shape"][0] for it in items])
    # warm-up: the first W requests served, and the smallest alone on the plain path
    if warm:
        serve_leg(capi, workloads, lib, warm, SAT_RATE, 1000 + rank, torch)
        plain_leg(capi, workloads, lib, [min(warm, key=lambda it: it["shape"][0])], torch)
    note("warm-up done")
    clocks = Clocks(local) if rank == 0 else None
    barrier(dist)
    # plain FP64, one request at a time
    t_plain, plain, prof = plain_leg(capi, workloads, lib, timed, torch)
    note("plain FP64 leg: %.1f s" % t_plain)
    # served, images in HBM
    barrier(dist)
    elapsed, served, failed, launches, _ = serve_leg(capi, workloads, lib, timed, SAT_RATE, 2000 + rank, torch)
    barrier(dist)
    elapsed = reduce_max(dist, elapsed)
    clk = clocks.stop() if clocks else None
    note("served leg: %.1f s" % elapsed)
    # end to end: pinned host images in, fields out
    sizes = [r["sizes"] for r in plain]
    e2e_elapsed, e2e_failed = None, None
    if not args.no_e2e:
        barrier(dist)
        e2e_elapsed, _, e2e_failed, _, _ = serve_leg(capi, workloads, lib, timed, SAT_RATE, 2000 + rank, torch,
                                                     resident=False, keep_fields=True, sizes=sizes)
        e2e_elapsed = reduce_max(dist, e2e_elapsed)
        note("end-to-end leg: %.1f s" % e2e_elapsed)
    value = world * K / elapsed
    plain_rate = K / t_plain
    errs = [abs(s["K"] - p["K"]) / abs(p["K"]) if (s and p["K"] != 0) else None for s, p in zip(served, plain)]
    valid = [e for e in errs if e is not None]
    p50, p99 = latency_stats(served)
    peak, peak_kind = load_peaks()
    achieved = LOOP_BYTES_PER_ROW * prof["rows"] / (prof["ms"] * 1e-3) / 1e9 if prof["ms"] > 0 else 0.0
    traffic = ncu_traffic()
    cells = sum(p["sizes"][0] * (p["outer_iterations"] + 1) for p in plain)
    if rank == 0:
        sweep = None
        if args.sweep and world == 1:
            sweep = {}
            nxt = args.first + W + K
            for q, rate in enumerate(SWEEP_RATES):
                seg = [materialize(capi, lib, workloads.stream_request(nxt + j), torch, dev)
                       for j in range(args.sweep_requests)]
                nxt += args.sweep_requests
                el, recs, fl, _, _ = serve_leg(capi, workloads, lib, seg, rate, 3000 + q, torch)
                a, b = latency_stats(recs)
                sweep["rate_%g" % rate] = {"arrival_rate_per_s": rate, "requests": len(seg), "failed": fl,
                                           "solves_per_s": (len(seg) - fl) / el, "p50_latency_s": a,
                                           "p99_latency_s": b, "edges": [it["shape"][0] for it in seg]}
                del seg
                note("sweep rate %g: %.1f s" % (rate, el))
        cpu, sphere64 = None, None
        if args.cpu_baseline and world == 1:
            sphere64 = {"gpu_plain_fp64": gpu_sphere64(capi, workloads, lib)}
            cores = physical_cores()
            o = oracle_complete_solve(cores)
            sphere64["cpu_oracle_%d_threads" % cores] = o
            if args.cpu_4_threads:
                try:
                    sphere64["cpu_oracle_4_threads"] = oracle_complete_solve(4)
                except Exception as e:  # a reported extra: it never stops the benchmark line
                    sphere64["cpu_oracle_4_threads"] = {"failed": str(e)[:200]}
            sphere64["gpu_speedup_vs_cpu_oracle"] = o["seconds"] / sphere64["gpu_plain_fp64"]["seconds"]
            sphere64["K_rel_diff_gpu_vs_oracle"] = abs(sphere64["gpu_plain_fp64"]["K"] - o["K"]) / abs(o["K"])
            note("cpu baseline: %.1f s on %d threads" % (o["seconds"], cores))
            cpu = {"value": 1.0 / o["seconds"], "unit": "solves/s", "cores": cores, "kind": "port",
                   "sample": "complete CPU-oracle solves of the 64^3 sphere pack (radius 6, porosity 0.55, SIMPLEC, "
                             "tolerances 1e-8, RMR < 1e-6; %d outer iterations, %.1f s) with %d OpenMP threads = "
                             "the host's physical cores; the GPU plain FP64 solve of the same case: %.2f s" % (
                                 o["outer_iterations"], o["seconds"], cores, sphere64["gpu_plain_fp64"]["seconds"])}
        readme64 = None
        if args.readme64 and world == 1:
            try:
                readme64 = run_readme64(capi, lib)
            except Exception as e:
                readme64 = {"error": repr(e)}
        batch64 = None
        if args.batch64 and world == 1:
            try:
                batch64 = run_batch64(capi, workloads, lib, torch, dev, args.batch64_images)
            except Exception as e:
                batch64 = {"error": repr(e)}
        large = run_large(capi, lib, args.large_outer) if (args.large and world == 1) else None
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1000.0 * elapsed / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "serving stream: Poisson arrivals at %g/s of permeability requests, cube images "
                                   "of edge log-uniform 48-192, sphere (r 3-8) or fibre (r 2-4) packs of porosity "
                                   "0.35-0.95 generated on the device, flow x/y/z, SIMPLEC or IDEAL; outer "
                                   "tolerance RMR < 1e-4, BiCGSTAB tolerances 1e-8" % SAT_RATE,
                       "requests": [describe(it) for it in timed], "max_active": SERVE_ACTIVE,
                       "served_precision": "FP32 inner BiCGSTAB with multilevel pressure preconditioner in FP64 "
                                           "defect correction",
                       "global_batch": world * K, "seq_len": None, "parallelism": "replicas x%d" % world,
                       "l2": "inputs and each request's working set exceed the 129 MB L2 for edges above ~100; "
                             "no flush"},
            "p50_latency_s": p50, "p99_latency_s": p99, "failed": failed,
            "K_rel_err_vs_plain_fp64": {"max": max(valid) if valid else None, "all": errs,
                                        "within_1e-4": all(e is not None and e <= K_TOL for e in errs)},
            "plain_fp64": {"solves_per_s": plain_rate, "seconds": t_plain,
                           "per_request_s": [round(p["seconds"], 3) for p in plain],
                           "outer_iterations": [p["outer_iterations"] for p in plain],
                           "converged": [p["converged"] for p in plain],
                           "cell_updates_per_s": cells / t_plain},
            "speedup_vs_plain_fp64": value / (world * plain_rate),
            "served_outer_iterations": [s["outer_iterations"] if s else None for s in served],
            "e2e": {"value": None if e2e_elapsed is None else world * K / e2e_elapsed, "unit": "solves/s",
                    "h2d_bytes_per_step": int(sum(it["nbytes"] for it in timed) / K),
                    "d2h_bytes_per_step": int(sum(8 * sum(s) for s in sizes) / K), "failed": e2e_failed},
            "roofline": {"bound": "hbm", "kernel": "k_kr_loop (BiCGSTAB iterations of the pressure solves, "
                                                   "plain FP64 leg)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind,
                         "traffic": None if traffic is None else traffic * prof["rows"] / max(prof["launches"], 1),
                         "traffic_bytes_per_row_iteration": traffic,
                         "bytes_per_row_iteration": LOOP_BYTES_PER_ROW,
                         "fused_bytes_per_row_iteration": LOOP_FUSED_BYTES_PER_ROW,
                         "avg_launch_ms": prof["ms"] / max(prof["launches"], 1),
                         "row_iterations_per_launch": prof["rows"] / max(prof["launches"], 1),
                         "launches": prof["launches"],
                         "phase_us_per_iteration": [round(1e3 * m / max(prof["iters"], 1), 2)
                                                    for m in prof["phase_ms"]]},
            "gpu_launches": int(launches),
            "cpu_baseline": cpu,
            "sphere64": sphere64,
            "rate_sweep": sweep,
            "batch64": batch64,
            "readme_64": readme64,
            "large": large,
            "clocks": clk,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_case(args):
    """One solve of a named workload (ncu captures: a launch of the kernel of
    interest on a known size): the 64^3 or 128^3 sphere pack, SIMPLEC, or
    request `--request` of the serving stream, `--max-outer` outer
    iterations, in the given precision."""
    import ns3d_gb300
    from ns3d_gb300 import capi, synth, workloads
    lib = ns3d_gb300.lib()
    prec = {"fp64": 0, "mixed": 1, "mixed_mg": 2}[args.precision]
    if args.case == "stream":
        q = workloads.stream_request(args.request)
        img, _, _ = capi.generate_image(lib, q["kind"], q["shape"], q["radius"], q["porosity"], q["image_seed"])
        p = workloads.stream_params(capi, lib, q, prec, max_outer=args.max_outer)
    else:
        img, info = {"sphere64": workloads.sphere64, "sphere128": workloads.sphere128}[args.case]()
        p = workloads.solve_params(capi, lib, img.shape[0], "SIMPLEC", 1, prec, max_outer=args.max_outer)
    s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
    l0 = lib.ns3d_kernel_launches()
    t = time.perf_counter()
    r = s.solve()
    print(json.dumps({"case": args.case, "request": args.request if args.case == "stream" else None,
                      "precision": args.precision, "np": s.sizes.np, "K": r.K,
                      "outer_iterations": int(r.iterations), "krylov_iterations": int(r.krylov_iterations),
                      "launches": int(lib.ns3d_kernel_launches() - l0), "fallbacks": s.mixed_fallbacks(),
                      "seconds": time.perf_counter() - t}))
    s.close()
    return 0


def main():
    global SERVE_ACTIVE
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=12, help="timed requests of the stream")
    ap.add_argument("--warmup", type=int, default=3, help="requests served before the timed legs")
    ap.add_argument("--first", type=int, default=0,
                    help="index of the first request of the stream used (0; profiling runs pick small ones)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-cpu-4-threads", dest="cpu_4_threads", action="store_false",
                    help="skip the 4-thread CPU-oracle solve (the reference README's thread count; about a minute)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-sweep", dest="sweep", action="store_false", help="skip the arrival-rate sweep")
    ap.add_argument("--sweep-requests", type=int, default=SWEEP_REQUESTS)
    ap.add_argument("--serving-active", type=int, default=SERVE_ACTIVE, help="solves in flight at most")
    ap.add_argument("--no-readme64", dest="readme64", action="store_false",
                    help="skip the reference's published 64^3 four-method case")
    ap.add_argument("--batch64", action="store_true",
                    help="add the 64-image batch sample (streams, merged sets, lockstep; about four minutes)")
    ap.add_argument("--batch64-images", type=int, default=64)
    ap.add_argument("--large", action="store_true", help="add the 256^3 fibre-pack sample (opt-in)")
    ap.add_argument("--large-outer", type=int, default=LARGE_OUTER)
    ap.add_argument("--case", choices=["sphere64", "sphere128", "stream"],
                    help="profiling mode: one solve of this workload instead of the benchmark")
    ap.add_argument("--request", type=int, default=13, help="the stream request of --case stream")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "mixed_mg"])
    ap.add_argument("--max-outer", type=int, default=1)
    args = ap.parse_args()
    SERVE_ACTIVE = args.serving_active
    if args.case:
        return run_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
