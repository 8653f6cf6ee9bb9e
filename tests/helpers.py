"""Shared helpers of the test suite (CPU oracle vs CUDA library)."""
import json
import os

import numpy as np

from ns3d_gb300 import capi, synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_runs.json")


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def params(lib, **kw):
    base = dict(dx=1e-6, mu=1e-3, rho=1.0, p0=1.0, alpha=0.5, beta=1.0, vsolvertol=1e-8, psolvertol=1e-8,
                pcsolvertol=1e-8, simpletol=1e-6, maxitsolver=2000, maxitSIMPLE=2000, N1=2, N2=2)
    base.update(kw)
    return capi.default_params(lib, **base)


def spheres_params(lib, **kw):
    """Parameters of the reference's tests/test_spheres.ini and compare_algorithms.ini."""
    base = dict(dx=2e-6, dy=-1, dz=-1, mu=1e-3, rho=1e3, p0=1e5, gradp=1e2, alpha=0.8, beta=1.0,
                vsolvertol=1e-5, psolvertol=1e-6, pcsolvertol=1e-3, simpletol=1e-4, maxitsolver=500,
                maxitSIMPLE=30, N1=2, N2=2, porevalue=0, direction=1, border=0, method="SIMPLEC")
    base.update(kw)
    return capi.default_params(lib, **base)


def solver(lib, img, prm):
    return capi.Solver(lib, prm, synth.to_raw(img), img.shape)


def rsa_image(shape, radius, phi, seed):
    img, _ = synth.rsa_spheres(shape, radius, phi, seed)
    return img


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))
