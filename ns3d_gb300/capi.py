"""ctypes binding of the NS3D C-ABI (include/ns3d_capi.h).

The same binding drives any library that implements the header: the CUDA
library built in this package and, in the tests, the CPU oracle.  This is the
binding a Python caller of the reference's solver path would add; the cgo and
C++ forms are shown in INTEGRATION.md.
"""
import ctypes as C
import os

import numpy as np

NS3D_OK = 0
SUCCESS, NUMERICAL_ISSUE, NO_CONVERGENCE, INVALID_INPUT = 0, 1, 2, 3
ERR_ARG, ERR_OOM, ERR_CUDA, ERR_IO, ERR_PARSE, ERR_STATE, ERR_TIMEOUT, ERR_UNSUPPORTED = range(-1, -9, -1)
SIMPLEC, SIMPLER, SIMPLERR, IDEAL = 0, 1, 2, 3
FP64, MIXED, MIXED_MG = 0, 1, 2
SYS_U, SYS_V, SYS_W, SYS_P = 0, 1, 2, 3
METHODS = {"SIMPLEC": SIMPLEC, "SIMPLER": SIMPLER, "SIMPLERR": SIMPLERR, "IDEAL": IDEAL}


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dx", "dy", "dz", "mu", "rho", "p0", "gradp", "alpha", "beta",
        "vsolvertol", "psolvertol", "pcsolvertol", "simpletol", "deltaRMR")] + \
        [(n, C.c_int32) for n in (
            "maxitsolver", "maxitSIMPLE", "N1", "N2", "save_step",
            "porevalue", "direction", "border", "method", "precision")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Sizes(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("nx", "ny", "nz", "np", "nu", "nv", "nw", "reserved")]


class Result(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "K", "Q", "v_moy", "RMR", "normdiv", "reldiv", "velocityNorm", "maxdiv", "MaxDeltaV",
        "p_inlet", "p_outlet", "p0", "p1", "alpha", "beta", "pcmax", "pcmin", "pcnorm", "seconds")] + \
        [(n, C.c_int32) for n in ("iterations", "converged", "it_u", "it_v", "it_w", "it_p")] + \
        [("krylov_iterations", C.c_int64), ("krylov_rows", C.c_int64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Profile(C.Structure):
    _fields_ = [("launches", C.c_int64 * 6), ("ms", C.c_double * 6), ("rows", C.c_int64 * 6),
                ("total_launches", C.c_int64)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("info", C.c_int32), ("error", C.c_double)]


_P = C.POINTER
_d = _P(C.c_double)
_i32 = _P(C.c_int32)


class NS3DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ns3d error %d: %s" % (code, msg))
        self.code = code


def _declare(lib):
    sig = {
        "ns3d_abi_version": (C.c_int, []),
        "ns3d_backend_name": (C.c_char_p, []),
        "ns3d_last_error": (C.c_char_p, []),
        "ns3d_params_default": (None, [_P(Params)]),
        "ns3d_open": (C.c_int, [_P(Params), _P(C.c_uint8), C.c_int32, C.c_int32, C.c_int32, _P(C.c_void_p)]),
        "ns3d_get_sizes": (C.c_int, [C.c_void_p, _P(Sizes)]),
        "ns3d_get_index_arrays": (C.c_int, [C.c_void_p, _i32, _i32, _i32, _i32]),
        "ns3d_set_initial_fields": (C.c_int, [C.c_void_p, _d, _d, _d, _d]),
        "ns3d_get_fields": (C.c_int, [C.c_void_p, _d, _d, _d, _d]),
        "ns3d_set_fields": (C.c_int, [C.c_void_p, _d, _d, _d, _d]),
        "ns3d_get_field_images": (C.c_int, [C.c_void_p, _d, _d, _d, _d, _d]),
        "ns3d_set_output": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int32]),
        "ns3d_solve": (C.c_int, [C.c_void_p]),
        "ns3d_get_result": (C.c_int, [C.c_void_p, _P(Result)]),
        "ns3d_assemble_momentum": (C.c_int, [C.c_void_p]),
        "ns3d_assemble_pressure_correction": (C.c_int, [C.c_void_p, C.c_int32]),
        "ns3d_assemble_pressure": (C.c_int, [C.c_void_p, C.c_int32]),
        "ns3d_get_system": (C.c_int, [C.c_void_p, C.c_int32, _d, _i32, _d, _d]),
        "ns3d_solve_system": (C.c_int, [C.c_void_p, C.c_int32, _d, _d, C.c_double, C.c_int32, _P(SolveInfo)]),
        "ns3d_close": (C.c_int, [C.c_void_p]),
    }
    if hasattr(lib, "ns3d_set_profiling"):
        sig["ns3d_set_profiling"] = (C.c_int, [C.c_void_p, C.c_int32])
        sig["ns3d_get_profile"] = (C.c_int, [C.c_void_p, _P(Profile)])
    if hasattr(lib, "ns3d_kernel_launches"):
        sig["ns3d_kernel_launches"] = (C.c_int64, [])
    if hasattr(lib, "ns3d_mixed_fallbacks"):
        sig["ns3d_mixed_fallbacks"] = (C.c_int32, [C.c_void_p])
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_LIBS = {}


def load(path):
    """Load (once) a library implementing include/ns3d_capi.h."""
    path = os.path.abspath(path)
    if path not in _LIBS:
        if not os.path.exists(path):
            raise OSError("NS3D library not found: %s" % path)
        _LIBS[path] = _declare(C.CDLL(path))
    return _LIBS[path]


def _ptr(a, ct):
    return None if a is None else a.ctypes.data_as(_P(ct))


def default_params(lib, **kw):
    p = Params()
    lib.ns3d_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "method" and isinstance(v, str):
            v = METHODS[v.upper()]
        setattr(p, k, v)
    return p


class Solver:
    """One solver instance (the C handle) on a given library."""

    def __init__(self, lib, params, raw_xfastest, dims):
        """raw_xfastest: the image as a numpy array, or the integer address of
        nx*ny*nz bytes in host or device memory."""
        self.lib = lib
        self.params = params
        if isinstance(raw_xfastest, int):
            ptr = C.cast(C.c_void_p(raw_xfastest), _P(C.c_uint8))
        else:
            raw = np.ascontiguousarray(raw_xfastest, dtype=np.uint8).reshape(-1)
            assert raw.size == dims[0] * dims[1] * dims[2]
            ptr = _ptr(raw, C.c_uint8)
        h = C.c_void_p()
        self._check(lib.ns3d_open(C.byref(params), ptr, int(dims[0]), int(dims[1]), int(dims[2]), C.byref(h)))
        self.h = h
        s = Sizes()
        self._check(lib.ns3d_get_sizes(h, C.byref(s)))
        self.sizes = s

    def _check(self, rc):
        if rc < 0:
            raise NS3DError(rc, self.lib.ns3d_last_error().decode())
        return rc

    @property
    def shape(self):
        return (self.sizes.nx, self.sizes.ny, self.sizes.nz)

    def n(self, sys):
        s = self.sizes
        return (s.nu, s.nv, s.nw, s.np)[sys]

    def index_arrays(self):
        nx, ny, nz = self.shape
        p = np.empty((nx, ny, nz), np.int32)
        u = np.empty((nx + 1, ny, nz), np.int32)
        v = np.empty((nx, ny, nz), np.int32)
        w = np.empty((nx, ny, nz), np.int32)
        self._check(self.lib.ns3d_get_index_arrays(self.h, _ptr(p, C.c_int32), _ptr(u, C.c_int32),
                                                   _ptr(v, C.c_int32), _ptr(w, C.c_int32)))
        return p, u, v, w

    def set_initial_fields(self, p=None, u=None, v=None, w=None):
        a = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (p, u, v, w)]
        self._check(self.lib.ns3d_set_initial_fields(self.h, *[_ptr(x, C.c_double) for x in a]))

    def fields(self):
        s = self.sizes
        out = [np.empty(n, np.float64) for n in (s.np, s.nu, s.nv, s.nw)]
        self._check(self.lib.ns3d_get_fields(self.h, *[_ptr(x, C.c_double) for x in out]))
        return out

    def set_fields(self, p=None, u=None, v=None, w=None):
        a = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (p, u, v, w)]
        self._check(self.lib.ns3d_set_fields(self.h, *[_ptr(x, C.c_double) for x in a]))

    def field_images(self):
        nx, ny, nz = self.shape
        p = np.empty((nx, ny, nz)); u = np.empty((nx + 1, ny, nz))
        v = np.empty((nx, ny, nz)); w = np.empty((nx, ny, nz)); va = np.empty((nx, ny, nz, 3))
        self._check(self.lib.ns3d_get_field_images(self.h, *[_ptr(x, C.c_double) for x in (p, u, v, w, va)]))
        return p, u, v, w, va

    def set_output(self, directory, stem, write_fields=True):
        d = None if directory is None else str(directory).encode()
        self._check(self.lib.ns3d_set_output(self.h, d, stem.encode(), int(bool(write_fields))))

    def solve(self):
        self._check(self.lib.ns3d_solve(self.h))
        return self.result()

    def sweep(self, gradps, warm_start=False):
        """ns3d_solve_sweep: one solve per pressure gradient on this image."""
        g = np.ascontiguousarray(gradps, dtype=np.float64)
        res = (Result * len(g))()
        f = self.lib.ns3d_solve_sweep
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, _P(C.c_double), C.c_int32, C.c_int32, _P(Result)]
        self._check(f(self.h, _ptr(g, C.c_double), len(g), int(bool(warm_start)), res))
        return list(res)

    def result(self):
        r = Result()
        self._check(self.lib.ns3d_get_result(self.h, C.byref(r)))
        return r

    def mixed_fallbacks(self):
        """Mixed-precision pressure solves of the last solve redone in FP64."""
        return self.lib.ns3d_mixed_fallbacks(self.h)

    def assemble_momentum(self):
        self._check(self.lib.ns3d_assemble_momentum(self.h))

    def assemble_pressure_correction(self, simplec=True):
        self._check(self.lib.ns3d_assemble_pressure_correction(self.h, int(bool(simplec))))

    def assemble_pressure(self, relax=True):
        self._check(self.lib.ns3d_assemble_pressure(self.h, int(bool(relax))))

    def system(self, sys):
        n = self.n(sys)
        coef = np.empty((7, n)); nbr = np.empty((6, n), np.int32)
        rhs = np.empty(n); rs = np.empty(n)
        self._check(self.lib.ns3d_get_system(self.h, sys, _ptr(coef, C.c_double), _ptr(nbr, C.c_int32),
                                             _ptr(rhs, C.c_double), _ptr(rs, C.c_double)))
        return coef, nbr, rhs, rs

    def solve_system(self, sys, x, tol, maxit, rhs=None):
        x = np.ascontiguousarray(x, np.float64).copy()
        info = SolveInfo()
        b = None if rhs is None else np.ascontiguousarray(rhs, np.float64)
        self._check(self.lib.ns3d_solve_system(self.h, sys, _ptr(b, C.c_double), _ptr(x, C.c_double),
                                               float(tol), int(maxit), C.byref(info)))
        return x, info

    def set_profiling(self, enable=True):
        self._check(self.lib.ns3d_set_profiling(self.h, int(bool(enable))))

    def profile(self):
        p = Profile()
        self._check(self.lib.ns3d_get_profile(self.h, C.byref(p)))
        return p

    def close(self):
        if getattr(self, "h", None):
            self.lib.ns3d_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("active", C.c_int32), ("peak_active", C.c_int32),
                ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double), ("mean_latency_s", C.c_double),
                ("solves_per_s", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class GroupStats(C.Structure):
    """ns3d_group_stats: merged solve sets run, member sets and systems served."""
    _fields_ = [("launches", C.c_int64), ("requests", C.c_int64), ("systems", C.c_int64),
                ("max_systems", C.c_int32), ("max_requests", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def _declare_server(lib):
    if getattr(lib, "_ns3d_server_declared", False):
        return lib
    sig = {
        "ns3d_server_start": (C.c_int, [C.c_int32, C.c_size_t, _P(C.c_void_p)]),
        "ns3d_server_submit": (C.c_int, [C.c_void_p, _P(Params), _P(C.c_uint8), C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int32, _P(C.c_int64)]),
        "ns3d_server_submit_resident": (C.c_int, [C.c_void_p, _P(Params), C.c_void_p, C.c_int32, C.c_int32,
                                                  C.c_int32, C.c_int32, _P(C.c_int64)]),
        "ns3d_server_poll": (C.c_int, [C.c_void_p, C.c_int64, _P(C.c_int32), _P(Result)]),
        "ns3d_server_wait": (C.c_int, [C.c_void_p, C.c_int64, _P(Result), _P(C.c_double)]),
        "ns3d_server_fields": (C.c_int, [C.c_void_p, C.c_int64, _d, _d, _d, _d]),
        "ns3d_server_get_stats": (C.c_int, [C.c_void_p, _P(ServerStats)]),
        "ns3d_server_stop": (C.c_int, [C.c_void_p]),
        "ns3d_server_cancel_queued": (C.c_int, [C.c_void_p, _P(C.c_int64)]),
        "ns3d_batch_solve": (C.c_int, [_P(Params), _P(_P(C.c_uint8)), _i32, C.c_int32, C.c_int32, _P(Result),
                                       _i32]),
        "ns3d_batch_solve_merged": (C.c_int, [_P(Params), _P(_P(C.c_uint8)), _i32, C.c_int32, C.c_int32,
                                              C.c_int32, _P(Result), _i32, _P(GroupStats)]),
        "ns3d_server_set_merging": (C.c_int, [C.c_void_p, C.c_int32]),
        "ns3d_server_group_stats": (C.c_int, [C.c_void_p, _P(GroupStats)]),
        "ns3d_group_create": (C.c_int, [C.c_int32, _P(C.c_void_p)]),
        "ns3d_set_group": (C.c_int, [C.c_void_p, C.c_void_p]),
        "ns3d_group_get_stats": (C.c_int, [C.c_void_p, _P(GroupStats)]),
        "ns3d_group_destroy": (C.c_int, [C.c_void_p]),
        "ns3d_solve_lockstep": (C.c_int, [_P(C.c_void_p), C.c_int32, _i32]),
        "ns3d_batch_solve_lockstep": (C.c_int, [_P(Params), _P(_P(C.c_uint8)), _i32, C.c_int32, _P(Result), _i32]),
        "ns3d_autotune_enable": (C.c_int, [C.c_int32]),
        "ns3d_autotune_table": (C.c_int, [C.c_char_p, C.c_int32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._ns3d_server_declared = True
    return lib


class Server:
    """Continuous-batching solve server (ns3d_server_*)."""

    def __init__(self, lib, max_active, hbm_budget_bytes=0, merge=0):
        """merge: 0 no merging, n > 0 merged solve sets in a group of n lanes"""
        self.lib = _declare_server(lib)
        h = C.c_void_p()
        rc = self.lib.ns3d_server_start(int(max_active), int(hbm_budget_bytes), C.byref(h))
        if rc != 0:
            raise NS3DError(rc, "server start failed")
        self.h = h
        self.sizes = {}
        if merge:
            rc = self.lib.ns3d_server_set_merging(self.h, int(merge))
            if rc != 0:
                raise NS3DError(rc, "merging unavailable")

    def group_stats(self):
        g = GroupStats()
        self.lib.ns3d_server_group_stats(self.h, C.byref(g))
        return g

    def submit(self, params, raw_xfastest, dims, keep_fields=False):
        raw = np.ascontiguousarray(raw_xfastest, dtype=np.uint8).reshape(-1)
        t = C.c_int64()
        rc = self.lib.ns3d_server_submit(self.h, C.byref(params), _ptr(raw, C.c_uint8), int(dims[0]), int(dims[1]),
                                         int(dims[2]), int(bool(keep_fields)), C.byref(t))
        if rc != 0:
            raise NS3DError(rc, "submit failed")
        return t.value

    def submit_resident(self, params, raw_ptr, dims, keep_fields=False):
        """ns3d_server_submit_resident: `raw_ptr` (an integer address, host or
        device memory) is not copied and must stay valid until the request ends."""
        t = C.c_int64()
        rc = self.lib.ns3d_server_submit_resident(self.h, C.byref(params), C.c_void_p(int(raw_ptr)), int(dims[0]),
                                                  int(dims[1]), int(dims[2]), int(bool(keep_fields)), C.byref(t))
        if rc != 0:
            raise NS3DError(rc, "submit failed")
        return t.value

    def wait(self, ticket):
        r = Result()
        lat = C.c_double()
        rc = self.lib.ns3d_server_wait(self.h, int(ticket), C.byref(r), C.byref(lat))
        if rc != 0:
            raise NS3DError(rc, "request %d failed: %s" % (ticket, self.lib.ns3d_last_error().decode()))
        return r, lat.value

    def poll(self, ticket):
        st = C.c_int32()
        r = Result()
        rc = self.lib.ns3d_server_poll(self.h, int(ticket), C.byref(st), C.byref(r))
        return st.value, r, rc

    def fields(self, ticket, sizes):
        out = [np.empty(n, np.float64) for n in sizes]
        rc = self.lib.ns3d_server_fields(self.h, int(ticket), *[_ptr(x, C.c_double) for x in out])
        if rc != 0:
            raise NS3DError(rc, "fields of request %d unavailable" % ticket)
        return out

    def cancel_queued(self):
        n = C.c_int64()
        self.lib.ns3d_server_cancel_queued(self.h, C.byref(n))
        return n.value

    def stats(self):
        s = ServerStats()
        self.lib.ns3d_server_get_stats(self.h, C.byref(s))
        return s

    def stop(self):
        if getattr(self, "h", None):
            self.lib.ns3d_server_stop(self.h)
            self.h = None

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def generate_image(lib, kind, shape, radius, porosity, seed, max_prims=1 << 16):
    """ns3d_generate_image: a seeded sphere (kind 0) or fibre (kind 1) pack
    rasterised on the device.  Returns (image in C order (x, y, z), achieved
    porosity, primitives (k x 6))."""
    f = lib.ns3d_generate_image
    f.restype = C.c_int
    f.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_uint64, _P(C.c_uint8),
                  _P(C.c_double), _P(C.c_double), C.c_int32, _P(C.c_int32)]
    nx, ny, nz = (int(v) for v in shape)
    raw = np.empty(nx * ny * nz, np.uint8)
    prims = np.empty((max_prims, 6), np.float64)
    ach = C.c_double()
    k = C.c_int32()
    rc = f(int(kind), nx, ny, nz, int(radius), float(porosity), int(seed), _ptr(raw, C.c_uint8), C.byref(ach),
           _ptr(prims, C.c_double), int(max_prims), C.byref(k))
    if rc != 0:
        raise NS3DError(rc, lib.ns3d_last_error().decode())
    img = raw.reshape(nz, ny, nx).transpose(2, 1, 0).copy()
    return img, ach.value, prims[:min(k.value, max_prims)].copy()


class Group:
    """A solve group (ns3d_group_*): solver instances attached to it merge
    their FP64 BiCGSTAB sets into shared persistent launches while they solve
    on separate host threads."""

    def __init__(self, lib, lanes=1):
        self.lib = _declare_server(lib)
        h = C.c_void_p()
        rc = self.lib.ns3d_group_create(int(lanes), C.byref(h))
        if rc != 0:
            raise NS3DError(rc, lib.ns3d_last_error().decode())
        self.h = h

    def attach(self, solver):
        rc = self.lib.ns3d_set_group(solver.h, self.h)
        if rc != 0:
            raise NS3DError(rc, self.lib.ns3d_last_error().decode())

    def stats(self):
        g = GroupStats()
        self.lib.ns3d_group_get_stats(self.h, C.byref(g))
        return g

    def destroy(self):
        if getattr(self, "h", None):
            self.lib.ns3d_group_destroy(self.h)
            self.h = None


def batch_solve(lib, params_list, images_xfastest, dims_list, max_concurrent, merged=0):
    """ns3d_batch_solve / ns3d_batch_solve_merged (merged = lanes > 0) over host images.
    Returns (results, statuses, group stats or None, return code)."""
    lib = _declare_server(lib)
    n = len(params_list)
    raws = [np.ascontiguousarray(r, dtype=np.uint8).reshape(-1) for r in images_xfastest]
    ptrs = (_P(C.c_uint8) * n)(*[_ptr(r, C.c_uint8) for r in raws])
    dims = np.ascontiguousarray(np.array(dims_list, np.int32).reshape(-1))
    ps = (Params * n)(*params_list)
    res = (Result * n)()
    st = np.zeros(n, np.int32)
    if merged:
        g = GroupStats()
        rc = lib.ns3d_batch_solve_merged(ps, ptrs, _ptr(dims, C.c_int32), n, int(max_concurrent), int(merged),
                                         res, _ptr(st, C.c_int32), C.byref(g))
    else:
        g = None
        rc = lib.ns3d_batch_solve(ps, ptrs, _ptr(dims, C.c_int32), n, int(max_concurrent), res, _ptr(st, C.c_int32))
    return list(res), st, g, rc


def autotune_table(lib):
    """The merged-set grid autotuner's table (ns3d_autotune_table), one line
    per class of set."""
    lib = _declare_server(lib)
    buf = C.create_string_buffer(1 << 16)
    lib.ns3d_autotune_table(buf, len(buf))
    return buf.value.decode()


def solve_lockstep(lib, solvers):
    """ns3d_solve_lockstep: the solves of `solvers` (any mix of methods)
    driven together by this thread.  Returns (return code, per-solver
    statuses)."""
    lib = _declare_server(lib)
    n = len(solvers)
    hs = (C.c_void_p * n)(*[s.h.value for s in solvers])
    st = np.zeros(n, np.int32)
    rc = lib.ns3d_solve_lockstep(hs, n, _ptr(st, C.c_int32))
    return rc, st


def batch_solve_lockstep(lib, params_list, images_xfastest, dims_list):
    """ns3d_batch_solve_lockstep over host images: (results, statuses, return code)."""
    lib = _declare_server(lib)
    n = len(params_list)
    raws = [np.ascontiguousarray(r, dtype=np.uint8).reshape(-1) for r in images_xfastest]
    ptrs = (_P(C.c_uint8) * n)(*[_ptr(r, C.c_uint8) for r in raws])
    dims = np.ascontiguousarray(np.array(dims_list, np.int32).reshape(-1))
    ps = (Params * n)(*params_list)
    res = (Result * n)()
    st = np.zeros(n, np.int32)
    rc = lib.ns3d_batch_solve_lockstep(ps, ptrs, _ptr(dims, C.c_int32), n, res, _ptr(st, C.c_int32))
    return list(res), st, rc
