"""Lockstep solves: the solves of many images (different sizes, flow
directions, precisions and methods) driven together from one host thread --
every stage of an outer iteration for all images at once, the BiCGSTAB steps
as merged sets -- give each image exactly the result and the logs of its own
ns3d_solve."""
import numpy as np
import pytest

from helpers import params
from ns3d_gb300 import capi, synth, workloads

pytestmark = pytest.mark.gpu

# shape, radius, porosity, direction, precision
SPECS = [((20, 16, 18), 3, 0.6, 1, 0), ((24, 20, 16), 2, 0.7, 2, 0), ((16, 22, 20), 3, 0.55, 3, 0),
         ((18, 18, 24), 2, 0.65, 1, 1), ((22, 14, 20), 3, 0.6, 2, 2), ((28, 24, 22), 3, 0.6, 1, 2)]


def _requests(lib):
    reqs = []
    for k, (shape, r, phi, direction, precision) in enumerate(SPECS):
        img, _ = synth.rsa_spheres(shape, r, phi, seed=110 + k)
        # different outer-iteration caps: some images stop on the cap, others converge
        p = params(lib, method="SIMPLEC", direction=direction, precision=precision, maxitSIMPLE=40 + 20 * (k % 3),
                   simpletol=1e-5)
        reqs.append((p, img))
    return reqs


def _logs(d, direction):
    out = []
    for name in ("INFO-%d-case.log" % direction, "RES-%d-case.csv" % direction):
        out.append([x for x in (d / name).read_text().splitlines() if "terminated in" not in x])
    return out


def test_lockstep_equals_single_solves(gpulib, tmp_path):
    reqs = _requests(gpulib)
    alone = []
    for k, (p, img) in enumerate(reqs):
        d = tmp_path / ("a%d" % k)
        d.mkdir()
        s = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
        s.set_output(d, "case", False)
        r = s.solve()
        alone.append((r, s.fields(), _logs(d, p.direction)))
        s.close()
    solvers = []
    for k, (p, img) in enumerate(reqs):
        d = tmp_path / ("b%d" % k)
        d.mkdir()
        s = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
        s.set_output(d, "case", False)
        solvers.append(s)
    rc, st = capi.solve_lockstep(gpulib, solvers)
    assert rc == 0 and not st.any(), gpulib.ns3d_last_error()
    for k, (s, (ra, fa, la)) in enumerate(zip(solvers, alone)):
        r = s.result()
        for key in ("K", "RMR", "iterations", "converged", "it_u", "it_v", "it_w", "it_p", "krylov_iterations",
                    "alpha", "pcnorm"):
            assert getattr(r, key) == getattr(ra, key), (k, key)
        for a, b in zip(s.fields(), fa):
            assert np.array_equal(a, b), k
        assert _logs(tmp_path / ("b%d" % k), reqs[k][0].direction) == la, k
        s.close()


def test_lockstep_rejects_a_repeated_handle(gpulib):
    (p, img), = _requests(gpulib)[:1]
    a = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
    rc, st = capi.solve_lockstep(gpulib, [a, a])
    assert rc == capi.ERR_ARG and (st == capi.ERR_ARG).all()
    a.close()


# shape, radius, porosity, direction, precision, method, N1, N2
MIX = [((20, 16, 18), 3, 0.6, 1, 0, "SIMPLER", 2, 2), ((24, 20, 16), 2, 0.7, 2, 0, "SIMPLERR", 2, 2),
       ((16, 22, 20), 3, 0.55, 3, 0, "IDEAL", 2, 2), ((18, 18, 24), 2, 0.65, 1, 0, "IDEAL", 1, 3),
       ((22, 14, 20), 3, 0.6, 2, 0, "SIMPLEC", 2, 2), ((26, 18, 20), 3, 0.6, 1, 1, "IDEAL", 2, 2),
       ((20, 20, 20), 2, 0.65, 3, 2, "SIMPLER", 1, 2), ((28, 24, 22), 3, 0.6, 1, 2, "IDEAL", 2, 1),
       ((24, 22, 18), 3, 0.6, 2, 2, "SIMPLERR", 2, 2), ((22, 18, 26), 2, 0.6, 1, 2, "SIMPLEC", 2, 2)]


def _mix_requests(lib):
    reqs = []
    for k, (shape, r, phi, direction, precision, method, n1, n2) in enumerate(MIX):
        img, _ = synth.rsa_spheres(shape, r, phi, seed=150 + k)
        p = params(lib, method=method, direction=direction, precision=precision, maxitSIMPLE=30 + 15 * (k % 3),
                   simpletol=1e-5, N1=n1, N2=n2)
        reqs.append((p, img))
    return reqs


def _alone_then_lockstep(lib, reqs, tmp_path):
    alone = []
    for k, (p, img) in enumerate(reqs):
        d = tmp_path / ("a%d" % k)
        d.mkdir()
        s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
        s.set_output(d, "case", False)
        r = s.solve()
        alone.append((r, s.fields(), _logs(d, p.direction), s.mixed_fallbacks()))
        s.close()
    solvers = []
    for k, (p, img) in enumerate(reqs):
        d = tmp_path / ("b%d" % k)
        d.mkdir()
        s = capi.Solver(lib, p, synth.to_raw(img), img.shape)
        s.set_output(d, "case", False)
        solvers.append(s)
    rc, st = capi.solve_lockstep(lib, solvers)
    assert rc == 0 and not st.any(), lib.ns3d_last_error()
    for k, (s, (ra, fa, la, fb)) in enumerate(zip(solvers, alone)):
        r = s.result()
        for key in ("K", "RMR", "iterations", "converged", "it_u", "it_v", "it_w", "it_p", "krylov_iterations",
                    "krylov_rows", "alpha", "beta", "pcnorm", "normdiv", "velocityNorm"):
            assert getattr(r, key) == getattr(ra, key), (k, key)
        for a, b in zip(s.fields(), fa):
            assert np.array_equal(a, b), k
        assert _logs(tmp_path / ("b%d" % k), reqs[k][0].direction) == la, k
        assert s.mixed_fallbacks() == fb, k
        s.close()
    return alone


def test_lockstep_all_methods_equal_single_solves(gpulib, tmp_path):
    """SIMPLER, SIMPLER-R, IDEAL and SIMPLEC images with different N1/N2, in
    FP64, mixed precision and mixed precision with the multilevel
    preconditioner, in one lockstep call: each equals its own solve."""
    _alone_then_lockstep(gpulib, _mix_requests(gpulib), tmp_path)


def test_lockstep_redoes_failed_mixed_pressure_solves_in_fp64(gpulib, tmp_path):
    """Request 17 of the serving stream (74^3 fibres at porosity 0.36: many
    isolated pore clusters) stalls the FP32 pressure solves; its solve redoes
    them in FP64.  In lockstep, beside an IDEAL request, it takes the same
    fallback and gives the same bits."""
    reqs = []
    for i in (17, 11):
        q = workloads.stream_request(i)
        img, _, _ = capi.generate_image(gpulib, q["kind"], q["shape"], q["radius"], q["porosity"], q["image_seed"])
        reqs.append((workloads.stream_params(capi, gpulib, q, capi.MIXED_MG), img))
    alone = _alone_then_lockstep(gpulib, reqs, tmp_path)
    assert alone[0][3] > 0 and alone[0][0].converged == 1


def test_batch_lockstep_matches_single_solves(gpulib):
    reqs = _requests(gpulib)[:4]
    ks = []
    for p, img in reqs:
        s = capi.Solver(gpulib, p, synth.to_raw(img), img.shape)
        ks.append((s.solve().K, s.result().iterations))
        s.close()
    res, st, rc = capi.batch_solve_lockstep(gpulib, [p for p, _ in reqs], [synth.to_raw(img) for _, img in reqs],
                                            [img.shape for _, img in reqs])
    assert rc == 0 and not st.any()
    for r, (k, its) in zip(res, ks):
        assert r.K == k and r.iterations == its
