"""Pressure-drop sweeps on one image (ns3d_solve_sweep): cold starts equal
separate solves bit for bit; warm starts (the previous solution scaled by the
ratio of the pressure gradients, exact for Stokes flow) reach the same K in
fewer outer iterations."""
import numpy as np
import pytest

from helpers import params, solver
from ns3d_gb300 import synth

pytestmark = pytest.mark.gpu


def _gradients(shape):
    g0 = 1.0 / (shape[0] * 1e-6)
    return [g0, 2.0 * g0, 4.0 * g0]


@pytest.mark.parametrize("method", ["SIMPLEC", "IDEAL"])
def test_cold_sweep_equals_separate_solves(gpulib, method):
    img, _ = synth.rsa_spheres((20, 16, 18), 3, 0.6, seed=61)
    gs = _gradients(img.shape)
    s = solver(gpulib, img, params(gpulib, method=method, maxitSIMPLE=300, simpletol=1e-6, gradp=gs[0]))
    res = s.sweep(gs)
    s.close()
    for g, r in zip(gs, res):
        one = solver(gpulib, img, params(gpulib, method=method, maxitSIMPLE=300, simpletol=1e-6, gradp=g))
        r1 = one.solve()
        one.close()
        assert (r.K, r.iterations, r.p0, r.p1) == (r1.K, r1.iterations, r1.p0, r1.p1)


def test_warm_sweep_reaches_the_same_permeability_faster(gpulib):
    img, _ = synth.rsa_spheres((20, 16, 18), 3, 0.6, seed=62)
    gs = _gradients(img.shape)
    s = solver(gpulib, img, params(gpulib, maxitSIMPLE=400, simpletol=1e-7, gradp=gs[0]))
    cold = s.sweep(gs)
    warm = s.sweep(gs, warm_start=True)
    s.close()
    for c, w in zip(cold, warm):
        assert abs(w.K - c.K) <= 1e-4 * abs(c.K)
    assert sum(w.iterations for w in warm[1:]) < sum(c.iterations for c in cold[1:])
    # creeping flow: the permeability does not depend on the pressure drop
    assert abs(cold[2].K - cold[0].K) <= 1e-3 * abs(cold[0].K)


def test_warm_start_matches_oracle(gpulib, oracle):
    """The warm start of a sweep, checked against the oracle: the oracle
    solves the first gradient cold, its fields are scaled on the host exactly
    as the device scales them (u, v, w times the gradient ratio; p as
    p0_new + (p - p0_old) * ratio, the same roundings), and the oracle solves
    the second gradient from those fields.  The GPU sweep must give the same
    bits: result, outer iterations and fields."""
    img, _ = synth.rsa_spheres((20, 16, 18), 3, 0.6, seed=62)
    gs = _gradients(img.shape)[:2]
    kw = dict(maxitSIMPLE=400, simpletol=1e-7)
    s = solver(gpulib, img, params(gpulib, gradp=gs[0], **kw))
    warm = s.sweep(gs, warm_start=True)
    gpu_fields = s.fields()
    s.close()
    o0 = solver(oracle, img, params(oracle, gradp=gs[0], **kw))
    r0 = o0.solve()
    p, u, v, w = o0.fields()
    o0.close()
    assert (warm[0].K, warm[0].iterations) == (r0.K, r0.iterations)
    # p0 and p1 of the second solve, as the solver derives them (unit p0 here)
    p0_user, dx, nx = 1.0, 1e-6, img.shape[0]
    p1 = -gs[1] * (dx * nx) + p0_user
    p0_new = p0_user - p1 if p1 < 0 else p0_user
    ratio = gs[1] / gs[0]
    o1 = solver(oracle, img, params(oracle, gradp=gs[1], **kw))
    o1.set_fields(p0_new + (p - r0.p0) * ratio, u * ratio, v * ratio, w * ratio)
    r1 = o1.solve()
    ora_fields = o1.fields()
    o1.close()
    assert r1.p0 == p0_new
    assert (warm[1].K, warm[1].iterations, warm[1].RMR) == (r1.K, r1.iterations, r1.RMR)
    for a, b in zip(gpu_fields, ora_fields):
        assert np.array_equal(a, b)
