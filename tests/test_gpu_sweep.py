"""Pressure-drop sweeps on one image (ns3d_solve_sweep): cold starts equal
separate solves bit for bit; warm starts (the previous solution scaled by the
ratio of the pressure gradients, exact for Stokes flow) reach the same K in
fewer outer iterations."""
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
