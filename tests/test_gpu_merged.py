"""Merged solve sets: the BiCGSTAB sets (FP64, or FP32 inside FP64 defect
correction) of concurrent solves of different images (sizes, flow
directions, methods) run together in shared persistent loop-kernel launches
over a ragged list of chunks, and every solve gives exactly the result it
gives alone (bit-identical fields, K and iteration counts)."""
import threading

import numpy as np
import pytest

from helpers import params
from ns3d_gb300 import capi, synth

pytestmark = pytest.mark.gpu

SPECS = [((20, 16, 18), 3, 0.6, 1, "SIMPLEC"), ((24, 20, 16), 2, 0.7, 2, "IDEAL"),
         ((16, 22, 20), 3, 0.55, 3, "SIMPLEC"), ((18, 18, 24), 2, 0.65, 1, "SIMPLER"),
         ((22, 14, 20), 3, 0.6, 2, "SIMPLERR"), ((28, 24, 22), 3, 0.6, 1, "SIMPLEC")]


def _requests(lib, specs=SPECS):
    reqs = []
    for k, (shape, r, phi, direction, method) in enumerate(specs):
        img, _ = synth.rsa_spheres(shape, r, phi, seed=70 + k)
        p = params(lib, method=method, direction=direction, maxitSIMPLE=80, simpletol=1e-5)
        reqs.append((p, img))
    return reqs


def _alone(lib, reqs):
    out = []
    for p, img in reqs:
        s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
        r = s.solve()
        out.append((r.K, r.iterations, r.it_u, r.it_p, s.fields(), (s.sizes.np, s.sizes.nu, s.sizes.nv, s.sizes.nw)))
        s.close()
    return out


def _group_solve_and_compare(lib, reqs, lanes=1):
    """Solves every request alone, then all of them at once on their own
    threads with their solvers attached to one group; asserts bit-identical
    results and returns the group's statistics."""
    alone = _alone(lib, reqs)
    group = capi.Group(lib, lanes)
    solvers = [capi.Solver(lib, p, synth.to_raw(img), img.shape) for p, img in reqs]
    for s in solvers:
        group.attach(s)
    results = [None] * len(solvers)
    errors = []

    def work(i):
        try:
            results[i] = solvers[i].solve()
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(solvers))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for s, r, (k, its, it_u, it_p, fields, _) in zip(solvers, results, alone):
        assert r.K == k and r.iterations == its and r.it_u == it_u and r.it_p == it_p
        for a, b in zip(s.fields(), fields):
            assert np.array_equal(a, b)
    st = group.stats()
    for s in solvers:
        s.close()
    group.destroy()
    return st


@pytest.mark.parametrize("lanes", [1, 2])
def test_group_solves_equal_alone(gpulib, lanes):
    st = _group_solve_and_compare(gpulib, _requests(gpulib), lanes)
    # the sets were really merged: some launches served several solves
    assert st.launches > 0 and st.max_requests >= 2
    assert st.systems > st.launches
    if lanes == 2:  # cohorts of ceil(6 / 2) solves
        assert st.max_requests <= 3
    # the merged launches were timed for the grid autotuner (which may have
    # run them on different grids: the results above are bit-identical anyway)
    assert "kind=0" in capi.autotune_table(gpulib)


def test_group_detach_solves_alone(gpulib):
    """A solver attached and then detached (NULL group) solves on its own."""
    (p, img), = _requests(gpulib, SPECS[:1])
    (k, its, _, _, fields, _), = _alone(gpulib, [(p, img)])
    group = capi.Group(gpulib)
    s = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
    group.attach(s)
    assert capi._declare_server(gpulib).ns3d_set_group(s.h, None) == 0
    r = s.solve()
    assert r.K == k and r.iterations == its
    assert group.stats().launches == 0
    s.close()
    group.destroy()


def test_merged_batch_and_server_match_single_solves(gpulib):
    reqs = _requests(gpulib)[:4]
    alone = _alone(gpulib, reqs)
    res, status, g, rc = capi.batch_solve(gpulib, [p for p, _ in reqs], [synth.to_raw(img) for _, img in reqs],
                                          [img.shape for _, img in reqs], 4, merged=1)
    assert rc == 0 and not status.any()
    for r, (k, its, _, _, _, _) in zip(res, alone):
        assert r.K == k and r.iterations == its
    assert g.launches > 0 and g.max_requests >= 2

    srv = capi.Server(gpulib, max_active=4, merge=2)
    tickets = [srv.submit(p, synth.to_raw(img), img.shape, keep_fields=True) for p, img in reqs]
    for t, (k, its, _, _, fields, sizes) in zip(tickets, alone):
        r, lat = srv.wait(t)
        assert r.K == k and r.iterations == its and lat > 0
        for a, b in zip(srv.fields(t, sizes), fields):
            assert np.array_equal(a, b)
    gs = srv.group_stats()
    srv.stop()
    assert gs.launches > 0 and gs.requests >= len(reqs)


@pytest.mark.parametrize("precision", [1, 2], ids=["mixed", "mixed_mg"])
def test_mixed_precision_group_solves_equal_alone(gpulib, precision):
    """FP32-inner solves merge too (with the multilevel preconditioner of
    precision 2 applied per system inside the shared launch) and each gives
    its stand-alone result, bit for bit."""
    reqs = []
    for k, (shape, r_, phi, direction, method) in enumerate(SPECS[:4]):
        img, _ = synth.rsa_spheres(shape, r_, phi, seed=90 + k)
        reqs.append((params(gpulib, method=method, direction=direction, maxitSIMPLE=60, simpletol=1e-5,
                            precision=precision), img))
    st = _group_solve_and_compare(gpulib, reqs, lanes=2)
    assert st.launches > 0 and st.max_requests >= 2
