"""ns3d_bicgstab_noalloc: the BiCGSTAB entry point for callers that cannot
allocate device memory (hosts that run inside another framework's memory pool
or reserve all device memory up front, and hosts that forbid allocation after
start-up).  It keeps its work vectors in a fixed 65536-row device array inside
the library and allocates nothing per call.

Checked through the C-ABI against the existing entry point ns3d_solve_system on
the same assembled system, on two calls in a row (the second call reuses the
scratch left by the first).  Tolerance: the suite's bar, relative L2 <= 1e-8
and equal iteration counts (both entry points run the same kernels, so the
results are expected to be bit-identical as well).  This file is collected
last so that a failure here does not hide the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import params, rel_l2, solver
from ns3d_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.ns3d_bicgstab_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                  C.c_void_p, C.POINTER(capi.SolveInfo)]
    return f


def _device_system(torch, coef, nbr, rhs, n):
    npad = ((n + 1023) // 1024) * 1024
    c = np.zeros((7, npad))
    c[:, :n] = coef
    nb = np.full((6, npad), -1, np.int32)
    nb[:, :n] = nbr
    b = np.zeros(npad)
    b[:n] = rhs
    dev = torch.device("cuda:0")
    return (torch.from_numpy(c).to(dev), torch.from_numpy(nb).to(dev), torch.from_numpy(b).to(dev), npad)


def test_noalloc_matches_solve_system_twice(gpulib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    img, _ = synth.rsa_spheres((20, 16, 18), 3, 0.6, seed=31)
    s = solver(gpulib, img, params(gpulib, alpha=0.7))
    rng = np.random.default_rng(9)
    n = s.sizes
    s.set_fields(1.0 + 1e-3 * rng.standard_normal(n.np), 1e-6 * rng.standard_normal(n.nu),
                 1e-6 * rng.standard_normal(n.nv), 1e-6 * rng.standard_normal(n.nw))
    s.assemble_momentum()
    f = _noalloc(gpulib)
    stream = torch.cuda.current_stream().cuda_stream
    for call, sys in enumerate((capi.SYS_U, capi.SYS_V)):
        coef, nbr, rhs, _ = s.system(sys)
        m = s.n(sys)
        x0 = 1e-7 * rng.standard_normal(m)
        x_ref, info_ref = s.solve_system(sys, x0, 1e-10, 400)
        dc, dn, db, npad = _device_system(torch, coef, nbr, rhs, m)
        dx = torch.zeros(npad, dtype=torch.float64, device="cuda:0")
        dx[:m] = torch.from_numpy(x0).to("cuda:0")
        info = capi.SolveInfo()
        rc = f(dc.data_ptr(), dn.data_ptr(), db.data_ptr(), dx.data_ptr(), m, npad, 1e-10, 400, stream,
               C.byref(info))
        torch.cuda.synchronize()
        assert rc == 0, gpulib.ns3d_noalloc_last_error()
        x = dx[:m].cpu().numpy()
        assert info.iterations == info_ref.iterations and info.info == info_ref.info, call
        assert rel_l2(x, x_ref) <= 1e-8, call
        assert np.array_equal(x, x_ref), call


def test_noalloc_rejects_oversized_systems(gpulib):
    f = _noalloc(gpulib)
    info = capi.SolveInfo()
    rc = f(1, 1, 1, 1, 70000, 70656, 1e-8, 10, None, C.byref(info))
    assert rc == capi.ERR_ARG
