"""Failure paths on the GPU, in forms that fault, trap or hang nothing:

* the bounded grid barrier of the persistent solver kernels made to run out
  (every barrier waits for an arrival that never comes, with a 50 ms limit):
  the kernel stops, the solve returns NS3D_ERR_TIMEOUT, the context and the
  handle stay usable and the next solve gives the normal result bit for bit;
* geometries the reference handles with guards (src/NSBase.cxx:1950-1955 and
  the RMR division of src/SIMPLEC.cxx:150): a blocked outlet (no flow, K = 0,
  RMR not finite), a zero pressure drop (p_inlet == p_outlet, K = 0 by the
  guard) and a non-percolating image (a solid wall across the flow) -- the GPU
  path against the oracle;
* a NaN in a host input buffer, refused at the boundary.
"""
import ctypes
import math
import time

import numpy as np
import pytest

from helpers import params, solver
from ns3d_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _hook(lib):
    f = lib.ns3d_debug_barrier_timeout
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32, ctypes.c_double]
    return f


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED, capi.MIXED_MG])
def test_barrier_timeout_is_reported_and_recovered(gpulib, precision):
    img, _ = synth.rsa_spheres((24, 20, 18), 3, 0.6, seed=71)
    kw = dict(maxitSIMPLE=6, precision=precision)
    hook = _hook(gpulib)
    s = solver(gpulib, img, params(gpulib, **kw))
    try:
        assert hook(1, 0.05) == 0
        t = time.perf_counter()
        with pytest.raises(capi.NS3DError) as e:
            s.solve()
        elapsed = time.perf_counter() - t
    finally:
        assert hook(0, 0.0) == 0
    assert e.value.code == capi.ERR_TIMEOUT
    assert b"timed out" in gpulib.ns3d_last_error()
    assert elapsed < 10.0
    # the same handle, restarted from the default fields, solves normally
    s.set_initial_fields()
    r = s.solve()
    f = s.fields()
    s.close()
    fresh = solver(gpulib, img, params(gpulib, **kw))
    r1 = fresh.solve()
    f1 = fresh.fields()
    fresh.close()
    assert (r.K, r.iterations, r.RMR) == (r1.K, r1.iterations, r1.RMR)
    for a, b in zip(f, f1):
        assert np.array_equal(a, b)


def _same(a, b):
    return (math.isnan(a) and math.isnan(b)) or a == b


def _compare_with_oracle(gpulib, oracle, img, tmp_path, **kw):
    g = solver(gpulib, img, params(gpulib, **kw))
    o = solver(oracle, img, params(oracle, **kw))
    assert (g.sizes.np, g.sizes.nu, g.sizes.nv, g.sizes.nw) == (o.sizes.np, o.sizes.nu, o.sizes.nv, o.sizes.nw)
    for one, d in ((g, "g"), (o, "o")):
        (tmp_path / d).mkdir()
        one.set_output(str(tmp_path / d), "case", False)
    rg, ro = g.solve(), o.solve()
    for name in ("K", "Q", "v_moy", "RMR", "normdiv", "reldiv", "maxdiv", "MaxDeltaV", "p_inlet", "p_outlet"):
        assert _same(getattr(rg, name), getattr(ro, name)), name
    assert (rg.iterations, rg.converged, rg.it_p) == (ro.iterations, ro.converged, ro.it_p)
    for a, b in zip(g.fields(), o.fields()):
        assert np.array_equal(a, b, equal_nan=True)
    g.close()
    o.close()

    def lines(d, kind):
        text = (tmp_path / d / ("%s-1-case.%s" % (kind, "csv" if kind == "RES" else "log"))).read_text()
        # the sign a platform gives a NaN is not part of the result
        return [l.replace("-nan", "nan") for l in text.splitlines() if " terminated in " not in l]

    assert lines("g", "RES") == lines("o", "RES")
    assert lines("g", "INFO") == lines("o", "INFO")
    return rg


@pytest.mark.parametrize("method", ["SIMPLEC", "IDEAL"])
def test_blocked_outlet_matches_oracle(gpulib, oracle, tmp_path, method):
    img, _ = synth.rsa_spheres((20, 16, 14), 3, 0.65, seed=72)
    img[-1, :, :] = 1  # the outlet plane is solid: nothing flows out
    r = _compare_with_oracle(gpulib, oracle, img, tmp_path, method=method, maxitSIMPLE=5)
    assert r.K == 0.0 and r.v_moy == 0.0
    assert not math.isfinite(r.RMR)


def test_zero_pressure_drop_takes_the_permeability_guard(gpulib, oracle, tmp_path):
    img, _ = synth.rsa_spheres((20, 16, 14), 3, 0.65, seed=73)
    r = _compare_with_oracle(gpulib, oracle, img, tmp_path, gradp=0.0, maxitSIMPLE=5)
    assert r.p_inlet == r.p_outlet and r.K == 0.0


def test_non_percolating_image_matches_oracle(gpulib, oracle, tmp_path):
    img, _ = synth.rsa_spheres((20, 16, 14), 3, 0.65, seed=74)
    img[10, :, :] = 1  # a solid wall across the flow: two disconnected pore spaces
    _compare_with_oracle(gpulib, oracle, img, tmp_path, maxitSIMPLE=8)


def test_nan_in_host_field_refused(gpulib):
    img, _ = synth.rsa_spheres((16, 12, 10), 3, 0.65, seed=75)
    s = solver(gpulib, img, params(gpulib, maxitSIMPLE=3))
    p, u, v, w = s.fields()
    bad = p.copy()
    bad[len(bad) // 2] = np.nan
    with pytest.raises(capi.NS3DError) as e:
        s.set_fields(bad, u, v, w)
    assert e.value.code == capi.ERR_ARG
    nx, ny, nz = s.shape
    pimg = np.full((nx, ny, nz), 0.5)
    pimg[3, 4, 5] = np.inf
    with pytest.raises(capi.NS3DError) as e:
        s.set_initial_fields(p=pimg)
    assert e.value.code == capi.ERR_ARG
    # the refused calls changed nothing
    assert all(np.array_equal(a, b) for a, b in zip(s.fields(), (p, u, v, w)))
    s.close()
