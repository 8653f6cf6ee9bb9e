"""Seeded synthetic porous images (0 = fluid, 1 = solid), numpy only.

These stand in for the reference's image generator (src/gen_spheres.cxx,
a regular sphere lattice) and for the seeded workloads of the benchmark:
random sequential addition (RSA) sphere packs and isotropic random straight
fibres.  Images are returned in C order (x, y, z), z fastest -- the solver
frame; `to_raw` converts to the VTK file order (x fastest) that the C-ABI's
ns3d_open takes.
"""
import numpy as np


def to_raw(img):
    """C-order (x, y, z) image -> flat VTK-order buffer (x fastest)."""
    return np.ascontiguousarray(np.asarray(img, dtype=np.uint8).transpose(2, 1, 0)).reshape(-1)


def porosity(img):
    return float(1.0 - np.asarray(img, dtype=np.float64).mean())


def sphere_lattice(n, spacing, radius):
    """Regular lattice of spheres, centres at spacing/2 + spacing*m (the
    layout of MakeSphereLattice, src/gen_spheres.cxx:60-99)."""
    img = np.zeros((n, n, n), np.uint8)
    nper = n // spacing
    r2 = float(radius) * radius
    off = np.arange(-radius, radius + 1)
    d2 = off[:, None, None] ** 2 + off[None, :, None] ** 2 + off[None, None, :] ** 2
    ball = d2.astype(np.float64) <= r2
    for m in range(nper):
        for q in range(nper):
            for s in range(nper):
                c = np.array([spacing // 2 + spacing * m, spacing // 2 + spacing * q, spacing // 2 + spacing * s])
                _stamp(img, c, radius, ball)
    return img


def _stamp(img, c, radius, ball):
    lo = c - radius
    hi = c + radius + 1
    sl_img, sl_ball = [], []
    for a in range(3):
        l0, h0 = max(lo[a], 0), min(hi[a], img.shape[a])
        if l0 >= h0:
            return
        sl_img.append(slice(l0, h0))
        sl_ball.append(slice(l0 - lo[a], h0 - lo[a]))
    img[tuple(sl_img)] |= ball[tuple(sl_ball)].astype(np.uint8)


def _ball(radius):
    off = np.arange(-radius, radius + 1)
    d2 = off[:, None, None] ** 2 + off[None, :, None] ** 2 + off[None, None, :] ** 2
    return d2 <= radius * radius


def rsa_spheres(shape, radius, target_porosity, seed, overlap=False, max_failures=20000):
    """Random sequential addition of spheres until the porosity reaches the
    target.  Without overlap, a candidate centre closer than 2*radius to an
    accepted one is rejected.  Non-overlapping RSA jams near a solid fraction
    of ~0.38; when `max_failures` consecutive candidates are rejected the
    minimum centre distance is lowered by 10% (a seeded, documented fallback)
    so that denser targets are still reached.  Returns (image, info)."""
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape)
    img = np.zeros(shape, np.uint8)
    ball = _ball(radius)
    target_solid = 1.0 - target_porosity
    total = float(np.prod(shape))
    centres = []
    dmin = 0.0 if overlap else 2.0 * radius
    failures = 0
    relaxations = 0
    solid = 0
    while solid / total < target_solid:
        c = np.array([rng.integers(0, s) for s in shape])
        if dmin > 0 and centres:
            arr = np.asarray(centres)
            d2 = ((arr - c) ** 2).sum(axis=1)
            if d2.min() < dmin * dmin:
                failures += 1
                if failures >= max_failures:
                    dmin *= 0.9
                    relaxations += 1
                    failures = 0
                continue
        failures = 0
        centres.append(c)
        _stamp(img, c, radius, ball)
        solid = int(img.sum(dtype=np.int64))
    return img, {"porosity": porosity(img), "spheres": len(centres), "distance_relaxations": relaxations,
                 "min_centre_distance": dmin}


def random_fibres(shape, radius, target_porosity, seed):
    """Isotropic random straight solid fibres (infinite cylinders, overlap
    allowed).  Each fibre is drawn as the union of balls of `radius` centred
    every voxel along its axis; axes have uniformly random directions and pass
    through uniformly random points.  Returns (image, info)."""
    rng = np.random.default_rng(seed)
    shape = np.array(shape, dtype=np.int64)
    img = np.zeros(tuple(shape), np.uint8)
    ball = _ball(radius)
    total = float(np.prod(shape))
    L = float(np.sqrt((shape.astype(np.float64) ** 2).sum()))
    nf = 0
    while img.sum(dtype=np.int64) / total < 1.0 - target_porosity:
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        p = rng.uniform(0, 1, size=3) * shape
        for t in np.arange(-L, L, 1.0):
            c = np.rint(p + t * d).astype(np.int64)
            if np.all(c >= -radius) and np.all(c < shape + radius):
                _stamp(img, c, radius, ball)
        nf += 1
    return img, {"porosity": porosity(img), "fibres": nf}


def random_image(shape, fluid_fraction, seed):
    """Uncorrelated random voxels (edge cases and index-map tests)."""
    rng = np.random.default_rng(seed)
    return (rng.random(shape) >= fluid_fraction).astype(np.uint8)
