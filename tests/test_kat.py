"""Known-answer tests of the regularisation functions.

The scalar checks restate the reference's own tests (reference
test/testvortfunc.h:34-68) against the host function pointers the library
returns from cvtx_VortFunc_*; the table checks compare every function on a
grid of rho with values produced by the reference library (tests/golden/kat.npz).
"""
import math

import numpy as np
import pytest

import oracle
from conftest import REGS, golden


def test_reference_kats(cv):
    lib = cv.lib
    vfs = lib.cvtx_VortFunc_singular()
    assert vfs.g_3D(0.1) == 1.0 and vfs.g_3D(3.0) == 1.0
    assert vfs.zeta_3D(0.1) == 0.0 and vfs.zeta_3D(10.0) == 0.0
    vfw = lib.cvtx_VortFunc_winckelmans()
    assert vfw.g_3D(0.0) == 0.0
    assert abs(vfw.g_3D(1.0) - np.float32(0.61872)) < 1e-5
    assert abs(vfw.g_3D(10.0) - np.float32(0.9998168)) < 1e-7
    assert vfw.zeta_3D(0.0) == 7.5
    assert abs(vfw.zeta_3D(10.0) - 7.2433e-7) < 1e-11
    vfp = lib.cvtx_VortFunc_planetary()
    assert vfp.g_3D(0.0) == 0.0 and vfp.g_3D(1.0) == 1.0 and vfp.g_3D(10.0) == 1.0
    assert vfp.zeta_3D(0.99) == 3.0 and vfp.zeta_3D(1.01) == 0.0
    vfg = lib.cvtx_VortFunc_gaussian()
    assert vfg.g_3D(0.0) == 0.0
    for rho, val in [(0.5, 0.030859595), (1.0, 0.198748043), (2.0, 0.738535870),
                     (4.0, 0.998866015), (6.0, 0.999999925), (8.0, 0.999999999)]:
        assert abs(vfg.g_3D(rho) - val) < 1e-6, rho
    assert vfg.g_3D(10.0) == 1.0
    assert abs(vfg.zeta_3D(1.0) - 0.483941449) < 1e-6
    assert abs(vfg.zeta_3D(0.5) - 0.70413065) < 1e-6


@pytest.mark.parametrize("reg", REGS)
def test_regfuncs_match_reference_table(cv, reg):
    g = golden("kat")
    vf = getattr(cv.lib, f"cvtx_VortFunc_{reg}")()
    for which, fn in (("g3", vf.g_3D), ("g2", vf.g_2D), ("zeta3", vf.zeta_3D)):
        mine = np.array([fn(float(r)) for r in g["rho"]], np.float32)
        np.testing.assert_array_equal(mine, g[f"{which}_{reg}"], err_msg=f"{which} {reg}")
        orc = np.array([oracle.regfunc(reg, which, float(r)) for r in g["rho"]], np.float32)
        np.testing.assert_array_equal(orc, g[f"{which}_{reg}"], err_msg=f"oracle {which} {reg}")
    if reg in ("winckelmans", "gaussian"):
        for which, fn in (("eta3", vf.eta_3D), ("eta2", vf.eta_2D)):
            mine = np.array([fn(float(r)) for r in g["rho"]], np.float32)
            np.testing.assert_array_equal(mine, g[f"{which}_{reg}"], err_msg=f"{which} {reg}")
    tag = bytes(vf.cl_kernel_name_ext).split(b"\0")[0]
    assert tag == bytes(g[f"tag_{reg}"]).split(b"\0")[0] == reg.encode()


def test_redistfuncs(cv):
    lib = cv.lib
    for name, radius, probes in [
        ("lambda0", 0.5, [(0.2, 1.0), (0.7, 0.0)]),
        ("lambda1", 1.0, [(0.25, 0.75), (1.5, 0.0)]),
        ("lambda2", 1.5, [(0.25, 1 - 0.0625), (1.0, 0.0), (2.0, 0.0)]),
        ("lambda3", 2.0, [(0.5, 0.5 * 0.75 * 1.5), (1.5, (1 / 6) * -0.5 * 0.5 * 1.5)]),
        ("m4p", 2.0, [(0.5, 1 - 2.5 * 0.25 + 1.5 * 0.125), (1.5, 0.5 * -0.5 * 0.25)]),
    ]:
        rf = getattr(lib, f"cvtx_RedistFunc_{name}")()
        assert rf.radius == radius
        for u, val in probes:
            assert math.isclose(rf.func(u), val, rel_tol=1e-6, abs_tol=1e-7), (name, u)
