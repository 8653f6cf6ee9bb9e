"""NS3D on GB300: steady staggered-grid Navier-Stokes permeability solver.

Host-side mirror of the reference's solver path (jerome-lux/NS3D): the same
ini keys, .vti inputs/outputs, SIMPLEC/SIMPLER/SIMPLERR/IDEAL outer loops and
RES/INFO logs, with every step of the outer loop running as hand-written
sm_103a kernels in ns3d_gb300/_lib/libns3d_gb300.so (C-ABI in
include/ns3d_capi.h).  There is no CPU fallback: when the library is missing
the calls below raise.
"""
import ctypes as _C
import os as _os

import numpy as _np

from . import capi
from .capi import NS3DError, Params, Result, Solver  # noqa: F401

_HERE = _os.path.dirname(_os.path.abspath(__file__))
LIB_PATH = _os.path.join(_HERE, "_lib", "libns3d_gb300.so")
EXE_PATH = _os.path.join(_HERE, "_lib", "NS3D")


def build(verbose=False):
    """Compile the CUDA library in-tree (sm_103a)."""
    from .build import build as _b
    return _b(verbose=verbose)


def lib():
    """The CUDA library; raises OSError when it has not been built."""
    if not _os.path.exists(LIB_PATH):
        raise OSError("libns3d_gb300.so is not built (run ns3d_gb300.build()); there is no CPU fallback")
    return capi.load(LIB_PATH)


def default_params(**kw):
    return capi.default_params(lib(), **kw)


def open_solver(params, image_c_order):
    """Solver instance on the GPU from a C-order (x, y, z) binary image."""
    img = _np.asarray(image_c_order, dtype=_np.uint8)
    raw = _np.ascontiguousarray(img.transpose(2, 1, 0)).reshape(-1)
    return Solver(lib(), params, raw, img.shape)


def read_ini(path):
    """ReadInput: (params, files dict)."""
    L = lib()
    p = Params()
    cap = 4096
    bufs = [_C.create_string_buffer(cap) for _ in range(5)]
    L.ns3d_ini_read.restype = _C.c_int
    L.ns3d_ini_read.argtypes = [_C.c_char_p, _C.POINTER(Params)] + [_C.c_char_p] * 5 + [_C.c_size_t]
    rc = L.ns3d_ini_read(str(path).encode(), _C.byref(p), *bufs, cap)
    if rc != 0:
        raise NS3DError(rc, "cannot read ini file %s" % path)
    keys = ("input", "pressurefield", "vxfield", "vyfield", "vzfield")
    return p, {k: b.value.decode() for k, b in zip(keys, bufs)}


def read_vti_u8(path):
    """Voxel image of a .vti/.vtk file, C order (x, y, z)."""
    L = lib()
    dims = (_C.c_int32 * 3)()
    L.ns3d_vti_read_u8.argtypes = [_C.c_char_p, _C.c_void_p, _C.c_size_t, _C.POINTER(_C.c_int32)]
    rc = L.ns3d_vti_read_u8(str(path).encode(), None, 0, dims)
    if rc != 0:
        raise NS3DError(rc, "cannot read %s" % path)
    n = dims[0] * dims[1] * dims[2]
    buf = _np.empty(n, _np.uint8)
    rc = L.ns3d_vti_read_u8(str(path).encode(), buf.ctypes.data, n, dims)
    if rc != 0:
        raise NS3DError(rc, "cannot read %s" % path)
    return buf.reshape(dims[2], dims[1], dims[0]).transpose(2, 1, 0).copy()


def read_vti_f64(path):
    """Field of a .vti file, C order (x, y, z[, comp])."""
    L = lib()
    dims = (_C.c_int32 * 3)()
    nc = _C.c_int32()
    L.ns3d_vti_read_f64.argtypes = [_C.c_char_p, _C.c_void_p, _C.c_size_t, _C.POINTER(_C.c_int32),
                                    _C.POINTER(_C.c_int32)]
    rc = L.ns3d_vti_read_f64(str(path).encode(), None, 0, dims, _C.byref(nc))
    if rc != 0:
        raise NS3DError(rc, "cannot read %s" % path)
    n = dims[0] * dims[1] * dims[2] * nc.value
    buf = _np.empty(n, _np.float64)
    rc = L.ns3d_vti_read_f64(str(path).encode(), buf.ctypes.data, n, dims, _C.byref(nc))
    if rc != 0:
        raise NS3DError(rc, "cannot read %s" % path)
    if nc.value == 1:
        return buf.reshape(dims[2], dims[1], dims[0]).transpose(2, 1, 0).copy()
    return buf.reshape(dims[2], dims[1], dims[0], nc.value).transpose(2, 1, 0, 3).copy()


def write_vti_f64(path, arr):
    L = lib()
    a = _np.ascontiguousarray(arr, dtype=_np.float64)
    nc = 1 if a.ndim == 3 else a.shape[3]
    L.ns3d_vti_write_f64.argtypes = [_C.c_char_p, _C.c_void_p] + [_C.c_int32] * 4
    rc = L.ns3d_vti_write_f64(str(path).encode(), a.ctypes.data, a.shape[0], a.shape[1], a.shape[2], nc)
    if rc != 0:
        raise NS3DError(rc, "cannot write %s" % path)


def write_vti_u8(path, img):
    L = lib()
    raw = _np.ascontiguousarray(_np.asarray(img, _np.uint8).transpose(2, 1, 0))
    L.ns3d_vti_write_u8.argtypes = [_C.c_char_p, _C.c_void_p] + [_C.c_int32] * 3
    rc = L.ns3d_vti_write_u8(str(path).encode(), raw.ctypes.data, img.shape[0], img.shape[1], img.shape[2])
    if rc != 0:
        raise NS3DError(rc, "cannot write %s" % path)


def run_ini(path, out_dir=None):
    """The NS3D program: solve the case described by an ini file."""
    L = lib()
    r = Result()
    L.ns3d_run_ini.argtypes = [_C.c_char_p, _C.c_char_p, _C.POINTER(Result)]
    rc = L.ns3d_run_ini(str(path).encode(), None if out_dir is None else str(out_dir).encode(), _C.byref(r))
    if rc != 0:
        raise NS3DError(rc, "NS3D run failed for %s" % path)
    return r
