"""The C-ABI boundary on CPU: the library loads, exports every symbol the
headers declare, keeps the reference's accelerator-API semantics, and its
host path (used when the caller disables every accelerator) reproduces the
reference. No GPU compute is called here."""
import ctypes as C
import platform
import re
import subprocess

import numpy as np
import pytest

from conftest import REGS, ROOT, golden
from cvortex_gb300 import abi
from oracle import exact


def _declared_symbols():
    names = []
    for h in sorted((ROOT / "include" / "cvortex").glob("*.h")):
        text = h.read_text()
        names += re.findall(r"CVTX_EXPORT\s+[^;(]*?\b(cvtx_\w+)\s*\(", text)
    return sorted(set(names))


def test_headers_declare_reference_abi():
    names = _declared_symbols()
    for n in abi.REFERENCE_SYMBOLS:
        assert n in names, n
    assert len([n for n in names if not n.startswith("cvtx_gb300_")]) == 52


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(str(abi.LIB_PATH))
    for name in _declared_symbols():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    assert exported == set(_declared_symbols()), exported ^ set(_declared_symbols())


def test_reference_test_program_passes_against_this_library(built):
    """The reference's own test program (test/testmain.c with its headers:
    regularisation KATs, particle directions and zeros, the accelerator
    API), compiled unchanged and linked against this libcvortex.so instead
    of the reference library, passes every test. Only where the reference
    sources are present; the binary goes to oracle/_ref/."""
    import oracle
    src = oracle.REFERENCE_ROOT / "test" / "testmain.c"
    if not src.is_file():
        pytest.skip("reference sources not present")
    out_dir = ROOT / "oracle" / "_ref"
    out_dir.mkdir(parents=True, exist_ok=True)
    exe = out_dir / "reference_testmain_gb300"
    lib_dir = abi.LIB_PATH.parent
    cmd = ["gcc", "-O2", "-fopenmp", "-w", "-I", str(ROOT / "include"),
           "-I", str(oracle.REFERENCE_ROOT / "include" / "cvortex"),
           "-I", str(oracle.REFERENCE_ROOT / "test"), "-DCVTX_EXPORT=", str(src), "-o", str(exe),
           "-L", str(lib_dir), "-lcvortex", "-lm", f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True, capture_output=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    m = re.search(r"Passed (\d+) of (\d+) tests \((\d+) failed\)", res.stdout)
    assert m and m.group(1) == m.group(2) and m.group(3) == "0", res.stdout[-2000:]
    assert int(m.group(2)) >= 57


def test_struct_layouts():
    assert C.sizeof(abi.cvtx_P3D) == 28
    assert C.sizeof(abi.cvtx_F3D) == 28
    assert C.sizeof(abi.cvtx_P2D) == 16
    assert C.sizeof(abi.cvtx_VortFunc) == 6 * C.sizeof(C.c_void_p) + 32


def test_accelerator_api_semantics(cv):
    """reference test/testaccelerators.h:35-67 (with its inverted expectation
    on the enable branch corrected)."""
    lib = cv.lib
    n = lib.cvtx_num_accelerators()
    assert 0 <= n < 64
    for i in range(n):
        assert lib.cvtx_accelerator_name(i) is not None
        was = lib.cvtx_accelerator_enabled(i)
        assert was in (0, 1)
        lib.cvtx_accelerator_disable(i)
        assert lib.cvtx_accelerator_enabled(i) == 0
        lib.cvtx_accelerator_enable(i)
        assert lib.cvtx_accelerator_enabled(i) == 1
        lib.cvtx_accelerator_enable(i)          # enabling twice is a no-op
        assert lib.cvtx_num_enabled_accelerators() <= n
    assert lib.cvtx_accelerator_name(n) is None
    assert lib.cvtx_accelerator_name(-1) is None
    info = lib.cvtx_information().decode()
    assert "cvortex version: 0.3.8" in info and "using CUDA: TRUE" in info


def test_initialise_finalise_cycle(built):
    c = abi.Cvtx()
    c.initialise()
    n = c.num_accelerators()
    assert c.lib.cvtx_num_enabled_accelerators() == (1 if n else 0)
    c.finalise()
    assert c.lib.cvtx_num_enabled_accelerators() == 0
    assert c.lib.cvtx_information() == b""
    c.initialise()
    c.initialise()    # repeat calls are harmless
    assert c.lib.cvtx_num_enabled_accelerators() == (1 if n else 0)


def test_particle_directions(cv):
    """Sign and zero pattern of single interactions (reference
    test/testparticle.h:33-112)."""
    lib = cv.lib
    V3 = abi.bsv_V3f

    def v(x, y, z):
        return V3((C.c_float * 3)(x, y, z))

    def p(c, w, vol=1.0):
        return abi.cvtx_P3D(v(*c), v(*w), vol)

    p1 = p((0, 0, 0), (1, 0, 0))
    for reg in ("winckelmans", "singular"):
        vf = getattr(lib, f"cvtx_VortFunc_{reg}")()
        r = lambda m: list(lib.cvtx_P3D_S2S_vel(C.byref(p1), m, C.byref(vf), 1.0).x)
        assert r(v(0, 0, 0)) == [0, 0, 0]
        assert r(v(1, 0, 0)) == [0, 0, 0]
        y, z, zbig = r(v(0, 1, 0)), r(v(0, 0, 1)), r(v(0, 0, 100))
        assert y[0] == 0 and y[1] == 0 and y[2] > 0
        assert z[0] == 0 and z[1] < 0 and z[2] == 0
        assert z[1] < zbig[1]
    vfs = lib.cvtx_VortFunc_singular()
    p2 = p((0, 0, 0), (0, 0, 1))
    d = lambda q: list(lib.cvtx_P3D_S2S_dvort(C.byref(p2), C.byref(q), C.byref(vfs), 1.0).x)
    a = d(p((0, 0, 1), (1, 0, 0)))
    assert a[0] == 0 and a[1] < 0 and a[2] == 0
    b = d(p((0, 0, 1), (0, 1, 0)))
    assert b[0] > 0 and b[1] == 0 and b[2] == 0
    assert d(p((0, 0, 1), (0, 0, 1))) == [0, 0, 0]


TOL = 0.0 if platform.machine() in ("x86_64", "AMD64") else 1e-6


def _close(a, b):
    if TOL == 0:
        np.testing.assert_array_equal(a, b)
    else:
        assert exact.rel_l2(a, b) <= TOL


@pytest.mark.parametrize("reg", REGS)
def test_host_path_matches_reference(host, reg):
    g = golden("p3d_ring")
    p, mes, s, nu = g["particles"], g["mes"], float(g["sigma"]), float(g["nu"])
    launches = host.launches()
    _close(host.p3d_vel(p, mes, reg, s), g[f"velmes_{reg}"])
    _close(host.p3d_dvort(p, p, reg, s, same=True), g[f"dvort_{reg}"])
    _close(host.p3d_visc(p, p, reg, s, nu, same=True), g[f"visc_{reg}"])
    _close(host.p3d_vort(p, mes, reg, s), g[f"vort_{reg}"])
    q = golden("p2d_patch")
    _close(host.p2d_vel(q["particles"], q["particles"]["coord"], reg, 0.05), q[f"vel_{reg}"])
    r = golden("relax")
    ring = r["particles"].copy()
    host.relax(ring, float(r["fdt"]), reg, float(r["sigma"]))
    _close(ring["vorticity"], r[f"vort_{reg}"])
    assert host.launches() == launches     # the host path launched nothing


def test_host_path_f3d(host):
    g = golden("f3d_sheet")
    f = g["filaments"]
    _close(host.f3d_vel(f, g["mes"]), g["vel"])
    _close(host.f3d_dvort(f, g["particles"]), g["dvort"])
    _close(host.f3d_inf_mtrx(f[:200], g["mes"][:40], g["dirs"]), g["inf"])


def test_zero_targets_is_a_noop(cv):
    p = golden("p3d_cube")["particles"]
    out = np.full((1, 3), 7.0, np.float32)
    ptrs = abi.ptr_array(p)
    cv.lib.cvtx_P3D_M2M_vel(ptrs.ctypes.data, len(p), out.ctypes.data, 0, out.ctypes.data,
                            C.byref(cv.vortfunc("winckelmans")), 0.05)
    assert np.all(out == 7.0)


def test_custom_regularisation_runs_host_function_pointers(cv):
    """A caller-built bundle with an empty tag is evaluated through its own
    function pointers (reference src/P3D.cpp:355), also with a GPU enabled."""
    vf = abi.cvtx_VortFunc()
    keep = abi.FN_F_F(lambda rho: 1.0)
    vf.g_3D = keep
    vf.cl_kernel_name_ext = b""
    p = golden("p3d_cube")["particles"][:50].copy()
    mes = golden("p3d_cube")["mes"][:20].copy()
    out = np.zeros((20, 3), np.float32)
    ptrs = abi.ptr_array(p)
    cv.lib.cvtx_P3D_M2M_vel(ptrs.ctypes.data, len(p), mes.ctypes.data, 20, out.ctypes.data,
                            C.byref(vf), 0.2)
    import oracle
    np.testing.assert_allclose(out, oracle.p3d_vel(p, mes, "singular", 0.2), rtol=1e-5, atol=1e-9)
