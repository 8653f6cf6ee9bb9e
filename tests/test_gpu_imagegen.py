"""Images generated on the device (ns3d_generate_image) against a CPU
rasterisation of the same primitives: equal voxel for voxel, and the number
of primitives is the smallest that reaches the target solid fraction."""
import numpy as np
import pytest

from ns3d_gb300 import capi

pytestmark = pytest.mark.gpu


def _ball(r):
    o = np.arange(-r, r + 1)
    return (o[:, None, None] ** 2 + o[None, :, None] ** 2 + o[None, None, :] ** 2) <= r * r


def _stamp(img, c, r, ball):
    lo = [int(v) - r for v in c]
    sl_i, sl_b = [], []
    for a in range(3):
        l0, h0 = max(lo[a], 0), min(lo[a] + 2 * r + 1, img.shape[a])
        if l0 >= h0:
            return
        sl_i.append(slice(l0, h0))
        sl_b.append(slice(l0 - lo[a], h0 - lo[a]))
    img[tuple(sl_i)] |= ball[tuple(sl_b)].astype(np.uint8)


def _raster(kind, shape, r, prims):
    img = np.zeros(shape, np.uint8)
    ball = _ball(r)
    shp = np.array(shape)
    L = float(np.sqrt((shp.astype(np.float64) ** 2).sum()))
    steps = int(np.ceil(2.0 * L))
    for q in prims:
        if kind == 0:
            _stamp(img, q[:3].astype(np.int64), r, ball)
            continue
        for s in range(steps):
            t = -L + float(s)
            c = np.rint(q[:3] + t * q[3:]).astype(np.int64)
            if np.all(c >= -r) and np.all(c < shp + r):
                _stamp(img, c, r, ball)
    return img


@pytest.mark.parametrize("kind,shape,radius,phi,seed", [(0, (40, 36, 32), 4, 0.6, 3), (1, (36, 40, 30), 2, 0.8, 9),
                                                         (0, (25, 31, 17), 3, 0.45, 11)])
def test_device_image_matches_cpu_rasterisation(gpulib, kind, shape, radius, phi, seed):
    img, ach, prims = capi.generate_image(gpulib, kind, shape, radius, phi, seed)
    assert img.shape == shape
    ref = _raster(kind, shape, radius, prims)
    assert np.array_equal(img, ref)
    assert ach == pytest.approx(1.0 - img.mean(), abs=0)
    # the smallest number of primitives that reaches the target
    assert 1.0 - img.mean() <= phi
    fewer = _raster(kind, shape, radius, prims[:-1])
    assert fewer.mean() < 1.0 - phi
    # the same seed gives the same image
    img2, _, _ = capi.generate_image(gpulib, kind, shape, radius, phi, seed)
    assert np.array_equal(img, img2)
