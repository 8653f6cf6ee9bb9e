"""GPU parity: the CUDA library against the CPU oracle, through the C-ABI.

Bar (stated per test): index arrays bit-exact; assembled systems, BiCGSTAB
iterates and full-solve fields/K bit-identical to the oracle (both follow the
same fixed reduction order and fused-multiply-add placement), which implies
the required |dK/K| <= 1e-8 and relative L2 field error <= 1e-8 -- those
tolerances are asserted too, so a failure says which bar broke.
"""
import numpy as np
import pytest

from helpers import params, rel_l2, solver, spheres_params
from ns3d_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL_K = 1e-8
TOL_FIELD = 1e-8

GEOMETRY_CASES = [
    # shape, fluid fraction, seed, direction, border, porevalue
    ((1, 1, 1), 1.0, 0, 1, 0, 0),
    ((2, 3, 4), 0.7, 1, 1, 0, 0),
    ((5, 1, 7), 0.8, 2, 1, 0, 0),
    ((7, 6, 1), 0.8, 3, 1, 0, 0),      # nz = 1: no w nodes
    ((13, 9, 11), 0.6, 4, 1, 0, 0),
    ((13, 9, 11), 0.6, 4, 2, 0, 0),    # rotation about z
    ((13, 9, 11), 0.6, 4, 3, 2, 0),    # rotation about y + border
    ((16, 16, 16), 0.3, 5, 1, 0, 0),   # mostly solid, many isolated cells
    ((16, 16, 16), 1.0, 6, 1, 1, 0),   # all fluid
    ((16, 16, 16), 0.0, 7, 1, 0, 0),   # all solid
    ((31, 17, 23), 0.55, 8, 1, 0, 1),  # porevalue 1 (voxels equal to 1 are fluid)
    ((40, 33, 37), 0.7, 9, 2, 3, 0),
]


def _image(shape, frac, seed, porevalue):
    img = synth.random_image(shape, frac, seed)
    return img if porevalue == 0 else (1 - img).astype(np.uint8)


@pytest.mark.parametrize("case", GEOMETRY_CASES, ids=lambda c: "x".join(map(str, c[0])) + "-d%d-b%d-pv%d" % c[3:])
def test_index_arrays_bit_exact(gpulib, oracle, case):
    shape, frac, seed, direction, border, pv = case
    img = _image(shape, frac, seed, pv)
    kw = dict(direction=direction, border=border, porevalue=pv)
    g = solver(gpulib, img, params(gpulib, **kw))
    o = solver(oracle, img, params(oracle, **kw))
    assert (g.sizes.nx, g.sizes.ny, g.sizes.nz, g.sizes.np, g.sizes.nu, g.sizes.nv, g.sizes.nw) == \
        (o.sizes.nx, o.sizes.ny, o.sizes.nz, o.sizes.np, o.sizes.nu, o.sizes.nv, o.sizes.nw)
    for a, b in zip(g.index_arrays(), o.index_arrays()):
        assert np.array_equal(a, b)


def test_index_arrays_lattice_128(gpulib, oracle):
    img = synth.sphere_lattice(128, 12, 5)
    g = solver(gpulib, img, spheres_params(gpulib))
    o = solver(oracle, img, spheres_params(oracle))
    assert (g.sizes.np, g.sizes.nu, g.sizes.nv, g.sizes.nw) == (1582152, 1517536, 1484768, 1484768)
    for a, b in zip(g.index_arrays(), o.index_arrays()):
        assert np.array_equal(a, b)


def _pair(gpulib, oracle, img, **kw):
    return solver(gpulib, img, params(gpulib, **kw)), solver(oracle, img, params(oracle, **kw))


def _random_fields(s, seed):
    rng = np.random.default_rng(seed)
    n = s.sizes
    return (1.0 + 1e-3 * rng.standard_normal(n.np), 1e-6 * rng.standard_normal(n.nu),
            1e-6 * rng.standard_normal(n.nv), 1e-6 * rng.standard_normal(n.nw))


def _systems_equal(g, o, sys):
    for a, b in zip(g.system(sys), o.system(sys)):
        assert np.array_equal(a, b), sys


@pytest.mark.parametrize("direction", [1, 3])
def test_assembly_bitwise(gpulib, oracle, direction):
    img, _ = synth.rsa_spheres((22, 18, 20), 3, 0.6, seed=11)
    g, o = _pair(gpulib, oracle, img, direction=direction, alpha=0.7, beta=0.9)
    f = _random_fields(g, 1)
    g.set_fields(*f)
    o.set_fields(*f)
    g.assemble_momentum()
    o.assemble_momentum()
    for sys in (capi.SYS_U, capi.SYS_V, capi.SYS_W):
        _systems_equal(g, o, sys)
    for simplec in (True, False):
        g.assemble_pressure_correction(simplec)
        o.assemble_pressure_correction(simplec)
        _systems_equal(g, o, capi.SYS_P)
    for relax in (True, False):
        g.assemble_pressure(relax)
        o.assemble_pressure(relax)
        _systems_equal(g, o, capi.SYS_P)


def test_bicgstab_bitwise(gpulib, oracle):
    img, _ = synth.rsa_spheres((24, 20, 22), 3, 0.55, seed=12)
    g, o = _pair(gpulib, oracle, img)
    f = _random_fields(g, 2)
    g.set_fields(*f)
    o.set_fields(*f)
    g.assemble_momentum()
    o.assemble_momentum()
    rng = np.random.default_rng(3)
    for sys in (capi.SYS_U, capi.SYS_V, capi.SYS_W):
        x0 = 1e-7 * rng.standard_normal(g.n(sys))
        xg, ig = g.solve_system(sys, x0, 1e-10, 500)
        xo, io = o.solve_system(sys, x0, 1e-10, 500)
        assert (ig.iterations, ig.info) == (io.iterations, io.info)
        assert ig.error == io.error
        assert np.array_equal(xg, xo)
    g.assemble_pressure_correction(True)
    o.assemble_pressure_correction(True)
    x0 = np.zeros(g.n(capi.SYS_P))
    xg, ig = g.solve_system(capi.SYS_P, x0, 1e-9, 2000)
    xo, io = o.solve_system(capi.SYS_P, x0, 1e-9, 2000)
    assert (ig.iterations, ig.info, ig.error) == (io.iterations, io.info, io.error)
    assert ig.iterations > 10 and ig.info == capi.SUCCESS
    assert np.array_equal(xg, xo)
    # iteration cap: NoConvergence with the iterate after `maxit` steps
    xg, ig = g.solve_system(capi.SYS_P, x0, 1e-14, 5)
    xo, io = o.solve_system(capi.SYS_P, x0, 1e-14, 5)
    assert ig.iterations == io.iterations == 5 and ig.info == io.info == capi.NO_CONVERGENCE
    assert np.array_equal(xg, xo)
    # zero right-hand side: x = 0, Success, iterations() reports the maximum
    z = np.zeros(g.n(capi.SYS_V))
    xg, ig = g.solve_system(capi.SYS_V, np.ones_like(z), 1e-8, 321, rhs=z)
    assert ig.iterations == 321 and ig.info == capi.SUCCESS and not xg.any()


def _compare_solves(g, o, tmp_path):
    g.set_output(tmp_path / "g", "case", False)
    o.set_output(tmp_path / "o", "case", False)
    rg = g.solve()
    ro = o.solve()
    for k in ("iterations", "converged", "it_u", "it_v", "it_w", "it_p", "krylov_iterations"):
        assert getattr(rg, k) == getattr(ro, k), k
    assert abs(rg.K - ro.K) <= TOL_K * abs(ro.K)
    for a, b in zip(g.fields(), o.fields()):
        assert rel_l2(a, b) <= TOL_FIELD
    # bit-identical: same reduction order and the same fused multiply-adds
    assert rg.K == ro.K and rg.RMR == ro.RMR
    for a, b in zip(g.fields(), o.fields()):
        assert np.array_equal(a, b)
    return rg, ro


@pytest.mark.parametrize("method", ["SIMPLEC", "SIMPLER", "SIMPLERR", "IDEAL"])
def test_full_solve_bitwise(gpulib, oracle, method, tmp_path):
    (tmp_path / "g").mkdir()
    (tmp_path / "o").mkdir()
    img, _ = synth.rsa_spheres((24, 16, 20), 3, 0.6, seed=21)
    g, o = _pair(gpulib, oracle, img, method=method, maxitSIMPLE=60, simpletol=1e-5)
    rg, _ = _compare_solves(g, o, tmp_path)
    assert rg.K > 0
    # the logs agree line for line except the wall-clock seconds
    for name in ("INFO-1-case.log", "RES-1-case.csv"):
        a = (tmp_path / "g" / name).read_text().splitlines()
        b = (tmp_path / "o" / name).read_text().splitlines()
        assert len(a) == len(b)
        for x, y in zip(a, b):
            if "terminated in" not in x:
                assert x == y


def test_direction_and_border_solve(gpulib, oracle, tmp_path):
    (tmp_path / "g").mkdir()
    (tmp_path / "o").mkdir()
    img, _ = synth.rsa_spheres((18, 22, 26), 3, 0.65, seed=22)
    g, o = _pair(gpulib, oracle, img, method="SIMPLEC", direction=3, border=2, maxitSIMPLE=12)
    _compare_solves(g, o, tmp_path)


def test_golden_config_first_iterations(gpulib, oracle, tmp_path):
    """tests/test_spheres.ini on the 128^3 lattice, 3 outer iterations."""
    (tmp_path / "g").mkdir()
    (tmp_path / "o").mkdir()
    img = synth.sphere_lattice(128, 12, 5)
    g = solver(gpulib, img, spheres_params(gpulib, maxitSIMPLE=3))
    o = solver(oracle, img, spheres_params(oracle, maxitSIMPLE=3))
    _compare_solves(g, o, tmp_path)


def test_initial_fields_and_images(gpulib, oracle):
    img, _ = synth.rsa_spheres((14, 12, 10), 2, 0.6, seed=23)
    g, o = _pair(gpulib, oracle, img)
    nx, ny, nz = g.shape
    rng = np.random.default_rng(5)
    pimg = rng.standard_normal((nx, ny, nz))
    uimg = rng.standard_normal((nx + 1, ny, nz))
    g.set_initial_fields(p=pimg, u=uimg)
    o.set_initial_fields(p=pimg, u=uimg)
    for a, b in zip(g.fields(), o.fields()):
        assert np.array_equal(a, b)
    for a, b in zip(g.field_images(), o.field_images()):
        assert np.array_equal(a, b)
