"""The seeded permeability workloads: images and solver parameters.

Shared by the benchmark and the parity tests so that both solve the same
inputs.  Every image is seeded synthetic data (no dataset is used); the
physics is the creeping-flow setting of the permeability solve: dx = 1e-6 m,
mu = 1e-3, rho = 1, a unit pressure drop along the flow axis (p0 = 1,
gradp = 1 / (extent * dx)), under-relaxation alpha = 0.5, beta = 1,
BiCGSTAB tolerances 1e-8 with at most 2000 iterations, outer convergence at a
relative mass residual below 1e-6.

  sphere64   64^3 non-overlapping RSA spheres, radius 6, porosity ~0.55,
             seed 0, SIMPLEC, flow x
  sphere128  128^3 non-overlapping RSA spheres, radius 8, porosity ~0.5,
             seed 1, flow x; SIMPLEC, SIMPLER (N1 = 2), SIMPLERR (N1 = 2),
             IDEAL (N1 = N2 = 2)
  fibre256   256^3 isotropic random straight fibres, radius 3, porosity
             ~0.85, seed 2, flow z

Non-overlapping random sequential addition jams near a solid fraction of
0.38; `synth.rsa_spheres` lowers the minimum centre distance by 10% after
20000 consecutive rejections so that porosity 0.5-0.55 is reached (the
achieved porosity is part of every record).
"""
import hashlib

import numpy as np

from . import synth

METHODS = ("SIMPLEC", "SIMPLER", "SIMPLERR", "IDEAL")
MAX_OUTER = 2000


def solve_params(capi, lib, extent, method="SIMPLEC", direction=1, precision=0, max_outer=MAX_OUTER, **kw):
    """ns3d_params of the creeping-flow permeability solve along `direction`
    (1 = x, 2 = y, 3 = z) with `extent` voxels along the flow."""
    dx = 1e-6
    base = dict(dx=dx, dy=-1.0, dz=-1.0, mu=1e-3, rho=1.0, p0=1.0, gradp=1.0 / (extent * dx),
                alpha=0.5, beta=1.0, vsolvertol=1e-8, psolvertol=1e-8, pcsolvertol=1e-8,
                simpletol=1e-6, maxitsolver=2000, maxitSIMPLE=max_outer, N1=2, N2=2, porevalue=0,
                direction=direction, border=0, method=method, precision=precision)
    base.update(kw)
    return capi.default_params(lib, **base)


def sphere64():
    """64^3 RSA spheres r = 6, porosity ~0.55, seed 0 (flow x, SIMPLEC)."""
    return synth.rsa_spheres((64, 64, 64), 6, 0.55, 0)


def sphere128():
    """128^3 RSA spheres r = 8, porosity ~0.5, seed 1 (flow x, four methods)."""
    return synth.rsa_spheres((128, 128, 128), 8, 0.5, 1)


def fibre256():
    """256^3 isotropic random fibres r = 3, porosity ~0.85, seed 2 (flow z)."""
    return synth.random_fibres((256, 256, 256), 3, 0.85, 2)


CASES = {
    "sphere64": {"image": sphere64, "direction": 1, "methods": ("SIMPLEC",)},
    "sphere128": {"image": sphere128, "direction": 1, "methods": METHODS},
}


def image_sha256(img):
    return hashlib.sha256(np.ascontiguousarray(img, dtype=np.uint8).tobytes()).hexdigest()


def field_sha256(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


# ---- the serving stream -------------------------------------------------------
# A seeded stream of permeability requests (request i from generator seed
# [STREAM_SEED, i]): a cube image of edge e, log-uniform in [48, 192]; a pack
# of overlapping spheres (radius 3-8 voxels) or of isotropic straight fibres
# (radius 2-4), porosity uniform in [0.35, 0.95], rasterised on the device
# (ns3d_generate_image); flow along x, y or z; SIMPLEC or IDEAL.  The
# physics is the creeping-flow setting above.  The numerics
# (STREAM_NUMERICS) take the outer-loop settings of the reference's own
# benchmark input (its tests/compare_algorithms.ini: alpha 0.8, convergence
# at RMR < 1e-4) and the linear-solver tolerances of the 64^3 case (1e-8, at
# most 2000 iterations): with tight inner solves, the plain FP64 and the
# mixed-precision solves of a request follow the same outer trajectory, so
# their K agree far inside 1e-4 (with the reference's loose inner tolerances,
# 1e-3 for the pressure correction, the two trajectories part and K differs
# by up to 3e-3 at RMR < 1e-4); the outer tolerance keeps the large
# high-porosity requests to hundreds of outer iterations.
STREAM_SEED = 4
STREAM_EDGE = (48, 192)
STREAM_NUMERICS = dict(alpha=0.8, vsolvertol=1e-8, psolvertol=1e-8, pcsolvertol=1e-8, simpletol=1e-4,
                       maxitsolver=2000)


def stream_request(i, seed=STREAM_SEED):
    """The i-th request of the serving stream: dict(shape, kind (0 spheres,
    1 fibres), radius, porosity (target), direction, method, image_seed)."""
    rng = np.random.default_rng([seed, i])
    e = int(round(float(np.exp(rng.uniform(np.log(STREAM_EDGE[0]), np.log(STREAM_EDGE[1]))))))
    kind = int(rng.integers(2))
    radius = int(rng.integers(3, 9)) if kind == 0 else int(rng.integers(2, 5))
    phi = float(rng.uniform(0.35, 0.95))
    direction = int(rng.integers(1, 4))
    method = ("SIMPLEC", "IDEAL")[int(rng.integers(2))]
    return {"index": i, "shape": (e, e, e), "kind": kind, "radius": radius, "porosity": phi,
            "direction": direction, "method": method, "image_seed": seed * 1000003 + i}


def stream_params(capi, lib, req, precision, max_outer=MAX_OUTER):
    """ns3d_params of a stream (or batch) request."""
    return solve_params(capi, lib, req["shape"][req["direction"] - 1], req["method"], req["direction"], precision,
                        max_outer=max_outer, **STREAM_NUMERICS)


# ---- many images at once ------------------------------------------------------
def batch64_request(i, seed=3):
    """Image i of the 64-image batch: each edge drawn from {32, 48, 64, 80, 96}
    per axis, a sphere pack (radius 3-8, porosity 0.35-0.9, overlap allowed)
    or a fibre pack (radius 2-4, porosity 0.7-0.95), flow along x, SIMPLEC."""
    rng = np.random.default_rng([seed, i])
    shape = tuple(int(rng.choice((32, 48, 64, 80, 96))) for _ in range(3))
    if rng.integers(2) == 0:
        kind, radius, phi = 0, int(rng.integers(3, 9)), float(rng.uniform(0.35, 0.9))
    else:
        kind, radius, phi = 1, int(rng.integers(2, 5)), float(rng.uniform(0.7, 0.95))
    return {"index": i, "shape": shape, "kind": kind, "radius": radius, "porosity": phi, "direction": 1,
            "method": "SIMPLEC", "image_seed": seed * 1000003 + i}
