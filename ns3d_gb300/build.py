"""Build recipe of the NS3D GB300 library (no cmake, a minute or two).

Compiles the CUDA translation units for sm_103a only (--fmad=false: the
arithmetic contract of the kernels; host code everywhere with
-ffp-contract=off, so the scalar control arithmetic on the host rounds as
written on x86-64 and on Arm alike), the host C++ files,
links libns3d_gb300.so in-tree under ns3d_gb300/_lib/ and the NS3D program
beside it.  Objects go to ns3d_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libns3d_gb300.so")
EXE = os.path.join(LIBDIR, "NS3D")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FILES = ["geometry.cu", "physics.cu", "krylov.cu", "solver.cu", "noalloc.cu", "mixed.cu", "mixed_host.cu", "imagegen.cu",
            "group.cu", "lockstep.cu"]
CPP_FILES = ["hostio.cpp", "capi_host.cpp", "serving.cpp", "tuner.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "ns3d_capi.h"))
    jobs = []
    objs = []
    for f in CU_FILES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "--extended-lambda",
                                   "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for f in CPP_FILES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall",
                         "-pthread",
                         "-I" + cuda_inc, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lz", "-lpthread", "-Xlinker", "-Bsymbolic"])
    main_src = os.path.join(CSRC, "main.cpp")
    if _stale(EXE, [main_src, LIB]):
        _run(["g++", "-O2", "-std=c++17", main_src, "-o", EXE, "-L" + LIBDIR, "-lns3d_gb300",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
