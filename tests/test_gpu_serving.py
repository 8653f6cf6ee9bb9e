"""Serving and batching: several solves of different sizes, directions and
methods admitted concurrently into one GPU give, for every request, exactly
the result it gives alone (bit-identical fields and K), and the server
reports its latency statistics."""
import numpy as np
import pytest

from helpers import params
from ns3d_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _requests(lib):
    reqs = []
    specs = [((20, 16, 18), 3, 0.6, 1, "SIMPLEC", 0), ((24, 20, 16), 2, 0.7, 2, "IDEAL", 0),
             ((16, 22, 20), 3, 0.55, 3, "SIMPLEC", 1), ((18, 18, 24), 2, 0.65, 1, "IDEAL", 1),
             ((22, 14, 20), 3, 0.6, 2, "SIMPLER", 0), ((26, 18, 14), 2, 0.7, 3, "SIMPLERR", 0)]
    for k, (shape, r, phi, direction, method, prec) in enumerate(specs):
        img, _ = synth.rsa_spheres(shape, r, phi, seed=50 + k)
        p = params(lib, method=method, direction=direction, precision=prec, maxitSIMPLE=80, simpletol=1e-5)
        reqs.append((p, img))
    return reqs


def test_each_result_is_the_same_alone_and_in_the_mix(gpulib):
    reqs = _requests(gpulib)
    alone = []
    for p, img in reqs:
        s = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
        r = s.solve()
        alone.append((r.K, r.iterations, s.fields(), (s.sizes.np, s.sizes.nu, s.sizes.nv, s.sizes.nw)))
        s.close()
    srv = capi.Server(gpulib, max_active=6)
    tickets = [srv.submit(p, synth.to_raw(img), img.shape, keep_fields=True) for p, img in reqs]
    for t, (k, its, fields, sizes) in zip(tickets, alone):
        r, lat = srv.wait(t)
        assert lat > 0
        assert r.K == k and r.iterations == its
        for a, b in zip(srv.fields(t, sizes), fields):
            assert np.array_equal(a, b)
    st = srv.stats()
    srv.stop()
    assert st.completed == len(reqs) and st.failed == 0
    assert st.peak_active >= 2
    assert 0 < st.p50_latency_s <= st.p99_latency_s


def test_admission_limit_and_continuous_admission(gpulib):
    """With max_active = 2, no more than two solves run at once, and requests
    submitted while others run are admitted as slots free up."""
    reqs = _requests(gpulib)[:4]
    srv = capi.Server(gpulib, max_active=2)
    tickets = [srv.submit(p, synth.to_raw(img), img.shape) for p, img in reqs[:2]]
    late = [srv.submit(p, synth.to_raw(img), img.shape) for p, img in reqs[2:]]
    for t in tickets + late:
        srv.wait(t)
    st = srv.stats()
    srv.stop()
    assert st.peak_active <= 2 and st.completed == 4


def test_batch_solve_matches_single_solves(gpulib):
    import ctypes as C
    reqs = _requests(gpulib)[:3]
    lib = capi._declare_server(gpulib)
    n = len(reqs)
    prm = (capi.Params * n)(*[p for p, _ in reqs])
    raws = [synth.to_raw(img) for _, img in reqs]
    ptrs = (C.POINTER(C.c_uint8) * n)(*[r.ctypes.data_as(C.POINTER(C.c_uint8)) for r in raws])
    dims = np.array([d for _, img in reqs for d in img.shape], np.int32)
    res = (capi.Result * n)()
    status = np.zeros(n, np.int32)
    rc = lib.ns3d_batch_solve(prm, ptrs, dims.ctypes.data_as(C.POINTER(C.c_int32)), n, 3, res,
                              status.ctypes.data_as(C.POINTER(C.c_int32)))
    assert rc == 0 and not status.any()
    for (p, img), r in zip(reqs, res):
        s = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
        assert s.solve().K == r.K
        s.close()


def test_hbm_budget_limits_admission(gpulib):
    """With an HBM budget below two requests' estimated footprint, the server
    runs one solve at a time although four slots are free; every request
    still completes."""
    reqs = _requests(gpulib)[:3]
    srv = capi.Server(gpulib, max_active=4, hbm_budget_bytes=1)
    tickets = [srv.submit(p, synth.to_raw(img), img.shape) for p, img in reqs]
    for t in tickets:
        r, _ = srv.wait(t)
        assert r.converged == 1 or r.iterations > 0
    st = srv.stats()
    srv.stop()
    assert st.peak_active == 1 and st.completed == 3


def test_cancel_queued_drops_only_waiting_requests(gpulib):
    reqs = _requests(gpulib)[:4]
    srv = capi.Server(gpulib, max_active=1)
    tickets = [srv.submit(p, synth.to_raw(img), img.shape) for p, img in reqs]
    import time
    deadline = time.time() + 30
    while srv.poll(tickets[0])[0] == 0 and time.time() < deadline:  # wait until the first is admitted
        time.sleep(0.01)
    n = srv.cancel_queued()
    states = [srv.poll(t)[0] for t in tickets]
    assert n >= 1 and states.count(3) == n
    r, _ = srv.wait(tickets[0])
    assert r.iterations > 0
    st = srv.stats()
    srv.stop()
    assert st.completed + n == 4 or st.completed >= 1
