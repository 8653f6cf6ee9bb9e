"""Host-side boundary: ini parsing (ReadInput semantics), .vti codec and the
C-ABI symbol table of both libraries.  No GPU needed."""
import ctypes
import os
import re

import numpy as np
import pytest

import ns3d_gb300 as ns
from ns3d_gb300 import capi, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ns3d_capi.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"NS3D_API\s+[\w\s\*]+?\b(ns3d_\w+)\s*\(", txt)))


def write(tmp_path, text, name="case.ini"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_header_declares_the_solver_surface():
    syms = declared_symbols()
    for s in ("ns3d_open", "ns3d_solve", "ns3d_get_result", "ns3d_get_index_arrays", "ns3d_run_ini",
              "ns3d_solve_system", "ns3d_get_system", "ns3d_close"):
        assert s in syms


def test_gpu_library_exports_every_declared_symbol(gpulib):
    for s in declared_symbols():
        assert hasattr(gpulib, s), s
    assert gpulib.ns3d_backend_name() == b"gb300"
    assert gpulib.ns3d_abi_version() == 1


def test_gpu_library_exports_nothing_undeclared(gpulib):
    """The C-ABI is exactly the header: no ns3d_ function leaves the library
    undeclared (everything else is hidden)."""
    import shutil
    import subprocess
    import ns3d_gb300
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-D", "--defined-only", ns3d_gb300.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert exported == set(declared_symbols())


def test_oracle_exports_the_solver_symbols(oracle):
    host_only = {"ns3d_ini_read", "ns3d_vti_read_u8", "ns3d_vti_read_f64", "ns3d_vti_write_f64",
                 "ns3d_vti_write_u8", "ns3d_run_ini", "ns3d_bicgstab_noalloc", "ns3d_noalloc_last_error",
                 "ns3d_set_profiling", "ns3d_get_profile", "ns3d_batch_solve", "ns3d_server_start",
                 "ns3d_server_submit", "ns3d_server_poll", "ns3d_server_wait", "ns3d_server_fields",
                 "ns3d_server_get_stats", "ns3d_server_stop", "ns3d_generate_image",
                 "ns3d_server_cancel_queued", "ns3d_solve_sweep", "ns3d_group_create", "ns3d_set_group",
                 "ns3d_group_get_stats", "ns3d_group_destroy", "ns3d_server_set_merging",
                 "ns3d_server_group_stats", "ns3d_batch_solve_merged", "ns3d_autotune_enable",
                 "ns3d_autotune_table", "ns3d_solve_lockstep", "ns3d_batch_solve_lockstep",
                 "ns3d_debug_barrier_timeout", "ns3d_server_submit_resident", "ns3d_kernel_launches",
                 "ns3d_mixed_fallbacks"}
    for s in declared_symbols():
        if s not in host_only:
            assert hasattr(oracle, s), s
    assert oracle.ns3d_backend_name() == b"oracle"


def test_params_defaults_match_reference(gpulib, oracle):
    # InputParams defaults, src/navierstokes3D.cxx:162-201
    for lib in (gpulib, oracle):
        p = capi.default_params(lib)
        assert (p.dx, p.dy, p.dz, p.mu, p.rho, p.p0, p.gradp) == (1.0, -1.0, -1.0, 1e-3, 1e3, 1e5, 1e2)
        assert (p.alpha, p.beta, p.vsolvertol, p.psolvertol, p.pcsolvertol, p.simpletol, p.deltaRMR) == \
            (0.8, 1.0, 1e-5, 1e-6, 1e-3, 1e-4, 1e-4)
        assert (p.maxitsolver, p.maxitSIMPLE, p.N1, p.N2, p.save_step, p.porevalue, p.direction, p.border) == \
            (1000, 500, 2, 2, 20, 0, 1, 0)


def test_ini_keys_case_comments_and_defaults(gpulib, tmp_path, capfd):
    path = write(tmp_path, """
# comment line
INPUT = img#1.vti   # file names may contain '#' without a space before it
dx = 2e-6
DY = -1
Mu=0.002
method = simpler    # case-insensitive
maxitSIMPLE = 7
N1 = 3
deltaRMR = 0.5
porevalue = 2
weird_key = 1
no equals sign here
""")
    p, files = ns.read_ini(path)
    err = capfd.readouterr().err
    assert files["input"] == "img#1.vti"
    assert files["pressurefield"] == "none"
    assert p.dx == 2e-6 and p.dy == 2e-6 and p.dz == 2e-6   # dy/dz <= 0 -> dx
    assert p.mu == 0.002 and p.method == capi.SIMPLER and p.maxitSIMPLE == 7 and p.N1 == 3
    # the reference lowercases keys but compares 'deltaRMR' in mixed case: never recognised
    assert p.deltaRMR == 1e-4 and "unknown key 'deltarmr'" in err
    assert p.porevalue == 0 and "'porevalue' should be 0 or 1" in err
    assert "unknown key 'weird_key'" in err and "no '=' found" in err


@pytest.mark.parametrize("text,msg", [
    ("dx = 1\n", "required key 'input'"),
    ("input = a.vti\nmu = abc\n", "expects a number"),
    ("input = a.vti\nmaxitsolver = 1.5\n", "expects a integer"),
    ("input = a.vti\ndirection = 4\n", "'direction' must be"),
    ("input = a.vti\nmethod = PISO\n", "unknown method"),
    ("input = a.vti\ndx = -1\n", "'dx' must be > 0"),
    ("input = a.vti\nsave_step = 0\n", "'save_step' must be > 0"),
    ("input =\n", "empty value"),
])
def test_ini_fatal_errors(gpulib, tmp_path, capfd, text, msg):
    path = write(tmp_path, text)
    with pytest.raises(capi.NS3DError) as e:
        ns.read_ini(path)
    assert e.value.code == capi.ERR_PARSE
    assert msg in capfd.readouterr().err


def test_ini_missing_file(gpulib, tmp_path):
    with pytest.raises(capi.NS3DError) as e:
        ns.read_ini(str(tmp_path / "nope.ini"))
    assert e.value.code == capi.ERR_IO


def test_vti_roundtrip_scalar_vector_u8(gpulib, tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((7, 5, 9))
    ns.write_vti_f64(tmp_path / "a.vti", a)
    assert np.array_equal(ns.read_vti_f64(tmp_path / "a.vti"), a)
    v = rng.standard_normal((4, 6, 3, 3))
    ns.write_vti_f64(tmp_path / "v.vti", v)
    assert np.array_equal(ns.read_vti_f64(tmp_path / "v.vti"), v)
    img = synth.random_image((9, 4, 6), 0.6, 1)
    ns.write_vti_u8(tmp_path / "i.vti", img)
    assert np.array_equal(ns.read_vti_u8(tmp_path / "i.vti"), img)
    # large enough for several 32 KiB compression blocks
    b = rng.standard_normal((40, 30, 20))
    ns.write_vti_f64(tmp_path / "b.vti", b)
    assert np.array_equal(ns.read_vti_f64(tmp_path / "b.vti"), b)


def test_vti_reads_uncompressed_and_ascii_and_legacy(gpulib, tmp_path):
    import base64, struct
    a = np.arange(2 * 3 * 4, dtype=np.float64).reshape(4, 3, 2)  # file order z, y, x
    c_order = a.transpose(2, 1, 0)
    head = '<?xml version="1.0"?>\n<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian" header_type="UInt32">\n' \
           '<ImageData WholeExtent="0 1 0 2 0 3" Origin="0 0 0" Spacing="1 1 1"><Piece Extent="0 1 0 2 0 3">' \
           '<PointData Scalars="s">'
    tail = '</PointData></Piece></ImageData>'
    payload = a.tobytes()
    enc = base64.b64encode(struct.pack("<I", len(payload))).decode() + base64.b64encode(payload).decode()
    (tmp_path / "app.vti").write_text(head + '<DataArray type="Float64" Name="s" format="appended" offset="0"/>' +
                                      tail + '<AppendedData encoding="base64">_' + enc + '</AppendedData></VTKFile>')
    assert np.array_equal(ns.read_vti_f64(tmp_path / "app.vti"), c_order)
    txt = " ".join(str(x) for x in a.reshape(-1))
    (tmp_path / "asc.vti").write_text(head + '<DataArray type="Float64" Name="s" format="ascii">' + txt +
                                      '</DataArray>' + tail + '</VTKFile>')
    assert np.array_equal(ns.read_vti_f64(tmp_path / "asc.vti"), c_order)
    img = synth.random_image((3, 4, 5), 0.5, 2)
    raw = synth.to_raw(img)
    leg = ("# vtk DataFile Version 3.0\nimg\nBINARY\nDATASET STRUCTURED_POINTS\nDIMENSIONS 3 4 5\n"
           "SPACING 1 1 1\nORIGIN 0 0 0\nPOINT_DATA 60\nSCALARS s unsigned_char 1\nLOOKUP_TABLE default\n").encode()
    (tmp_path / "leg.vtk").write_bytes(leg + raw.tobytes())
    assert np.array_equal(ns.read_vti_u8(tmp_path / "leg.vtk"), img)


def test_vti_errors(gpulib, tmp_path):
    with pytest.raises(capi.NS3DError) as e:
        ns.read_vti_u8(tmp_path / "missing.vti")
    assert e.value.code == capi.ERR_IO
    (tmp_path / "bad.vti").write_text("<VTKFile><ImageData WholeExtent='x'>")
    with pytest.raises(capi.NS3DError) as e:
        ns.read_vti_u8(tmp_path / "bad.vti")
    assert e.value.code == capi.ERR_PARSE
    # truncated compressed data
    img = synth.random_image((30, 30, 30), 0.5, 3)
    ns.write_vti_u8(tmp_path / "ok.vti", img)
    data = (tmp_path / "ok.vti").read_bytes()
    (tmp_path / "trunc.vti").write_bytes(data[: len(data) // 2])
    with pytest.raises(capi.NS3DError):
        ns.read_vti_u8(tmp_path / "trunc.vti")


def test_golden_fields_decode(gpulib):
    """The reference's golden outputs decode to the documented shapes (needs
    the reference checkout: its root in NS3D_REFERENCE_ROOT)."""
    root = os.environ.get("NS3D_REFERENCE_ROOT")
    if not root:
        pytest.skip("NS3D_REFERENCE_ROOT not set")
    ref = os.path.join(root, "tests", "results", "P-1-spheres_128.vti")
    p = ns.read_vti_f64(ref)
    assert p.shape == (128, 128, 128)
    u = ns.read_vti_f64(ref.replace("P-1", "Vx-1"))
    assert u.shape == (129, 128, 128)


def test_autotune_switch_and_empty_table(gpulib):
    """The merged-set autotuner's host interface: modes 0-2, the table of
    classes (empty before any merged launch), bad arguments rejected."""
    lib = capi._declare_server(gpulib)
    assert lib.ns3d_autotune_enable(3) == capi.ERR_ARG
    assert lib.ns3d_autotune_enable(2) == 0  # forget, stay on
    assert capi.autotune_table(gpulib) == ""
    assert lib.ns3d_autotune_table(None, 10) == capi.ERR_ARG
    assert lib.ns3d_autotune_enable(0) == 0 and lib.ns3d_autotune_enable(1) == 0


def test_lockstep_and_group_arguments_checked_without_work(gpulib):
    """The lockstep and group entry points check their arguments before any
    device work: NULL lists, negative counts and bad lane counts are
    rejected; an empty lockstep list is a no-op."""
    import ctypes as C
    lib = capi._declare_server(gpulib)
    assert lib.ns3d_solve_lockstep(None, 0, None) == 0
    assert lib.ns3d_solve_lockstep(None, 2, None) == capi.ERR_ARG
    assert lib.ns3d_solve_lockstep(None, -1, None) == capi.ERR_ARG
    hs = (C.c_void_p * 1)(None)
    st = np.full(1, 7, np.int32)
    assert lib.ns3d_solve_lockstep(hs, 1, st.ctypes.data_as(C.POINTER(C.c_int32))) == capi.ERR_ARG
    assert st[0] == capi.ERR_ARG
    res = (capi.Result * 1)()
    assert lib.ns3d_batch_solve_lockstep(None, None, None, 0, res, None) == capi.ERR_ARG
    g = C.c_void_p()
    assert lib.ns3d_group_create(0, C.byref(g)) == capi.ERR_ARG
    assert lib.ns3d_group_create(17, C.byref(g)) == capi.ERR_ARG
    assert lib.ns3d_group_create(1, None) == capi.ERR_ARG
    assert lib.ns3d_group_get_stats(None, None) == capi.ERR_ARG
    assert lib.ns3d_set_group(None, None) == capi.ERR_ARG


def test_non_finite_parameters_rejected_before_device_work(gpulib):
    """A NaN or an infinity in ns3d_params is refused by ns3d_open with
    NS3D_ERR_ARG before any device call (this runs without a GPU)."""
    raw = np.zeros(6 * 5 * 4, np.uint8)
    for name in ("dx", "dy", "mu", "rho", "p0", "gradp", "alpha", "beta", "pcsolvertol", "simpletol"):
        for bad in (float("nan"), float("inf"), -float("inf")):
            p = capi.default_params(gpulib, **{name: bad})
            h = ctypes.c_void_p()
            rc = gpulib.ns3d_open(ctypes.byref(p), raw.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), 6, 5, 4,
                                  ctypes.byref(h))
            assert rc == capi.ERR_ARG, (name, bad)
            assert b"not finite" in gpulib.ns3d_last_error(), name
            assert not h.value


def test_barrier_test_hook_arguments(gpulib):
    f = gpulib.ns3d_debug_barrier_timeout
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32, ctypes.c_double]
    assert f(-1, 1.0) == capi.ERR_ARG
    assert f(1, 0.0) == capi.ERR_ARG
    assert f(1, 11.0) == capi.ERR_ARG
    assert f(1, float("nan")) == capi.ERR_ARG
    assert f(0, 0.0) == 0
