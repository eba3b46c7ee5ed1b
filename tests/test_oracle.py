"""Pin the oracle: the C restatement of the reference CPU path against the
golden fixtures made by the reference library (tests/golden/make_golden.py),
against the reference library itself where it has been built, and the FP64
exact-math oracle against closed forms and the reference at moderate rho."""
import math

import numpy as np
import pytest

import oracle
from conftest import REGS, golden
from cvortex_gb300 import workloads
from oracle import exact


def _same(a, b, tol):
    if tol == 0:
        np.testing.assert_array_equal(a, b)
    else:
        assert exact.rel_l2(a, b) <= tol


# x86-64 builds of the restatement and the reference round identically (no FMA
# contraction); on other hosts allow the few-ulp differences of contracted FMAs.
import platform

TOL = 0.0 if platform.machine() in ("x86_64", "AMD64") else 1e-6


@pytest.mark.parametrize("case", ["cube", "ring"])
@pytest.mark.parametrize("reg", REGS)
def test_oracle_p3d_golden(built, case, reg):
    g = golden(f"p3d_{case}")
    p, mes, s, nu = g["particles"], g["mes"], float(g["sigma"]), float(g["nu"])
    _same(oracle.p3d_vel(p, p["coord"], reg, s), g[f"vel_{reg}"], TOL)
    _same(oracle.p3d_vel(p, mes, reg, s), g[f"velmes_{reg}"], TOL)
    _same(oracle.p3d_dvort(p, p, reg, s), g[f"dvort_{reg}"], TOL)
    _same(oracle.p3d_visc(p, p, reg, s, nu), g[f"visc_{reg}"], TOL)
    _same(oracle.p3d_vort(p, mes, reg, s), g[f"vort_{reg}"], TOL)


@pytest.mark.parametrize("reg", REGS)
def test_oracle_p2d_golden(built, reg):
    g = golden("p2d_patch")
    q, s, nu = g["particles"], float(g["sigma"]), float(g["nu"])
    _same(oracle.p2d_vel(q, q["coord"], reg, s), g[f"vel_{reg}"], TOL)
    # the reference sums this one with an OpenMP reduction (src/P2D.cpp:225)
    want = g[f"visc_{reg}"]
    got = oracle.p2d_visc(q, q, reg, s, nu)
    if np.any(want):
        assert exact.rel_l2(got, want) <= 1e-6
    else:
        assert not np.any(got)


def test_oracle_f3d_golden(built):
    g = golden("f3d_sheet")
    f = g["filaments"]
    _same(oracle.f3d_vel(f, g["mes"]), g["vel"], TOL)
    _same(oracle.f3d_dvort(f, g["particles"]), g["dvort"], TOL)
    _same(oracle.f3d_inf_mtrx(f[:200], g["mes"][:40], g["dirs"]), g["inf"], TOL)


def test_reference_comparison_inputs_regenerate():
    """The LCG restatement reproduces the stored first-repeat inputs of both
    reference comparison tests bit for bit."""
    import reftest_inputs as rt
    g = golden("reftest")
    ins = {(t, k): a for t, k, a in rt.all_inputs()}
    for test in ("single", "many"):
        a = ins[(test, 0)]
        for name in ("p3", "fil", "p2"):
            assert a[name].tobytes() == g[f"{test}_r0_{name}"].tobytes(), (test, name)


def test_oracle_reference_comparison_sections(built):
    """Every section of all 10 repeats of the reference's two comparison
    tests: the oracle against the reference library's CPU result, per
    element (bit for bit on x86-64 except P2D viscous, whose reference sum is
    an OpenMP reduction)."""
    import reftest_inputs as rt

    class _Oracle:
        p3d_vel = staticmethod(lambda s, m, r, sg: oracle.p3d_vel(s, m, r, sg))
        p3d_dvort = staticmethod(lambda s, t, r, sg, same=False: oracle.p3d_dvort(s, t, r, sg))
        p3d_visc = staticmethod(lambda s, t, r, sg, nu, same=False: oracle.p3d_visc(s, t, r, sg, nu))
        f3d_vel = staticmethod(oracle.f3d_vel)
        f3d_dvort = staticmethod(oracle.f3d_dvort)
        p2d_vel = staticmethod(lambda s, m, r, sg: oracle.p2d_vel(s, m, r, sg))
        p2d_visc = staticmethod(lambda s, t, r, sg, nu, same=False: oracle.p2d_visc(s, t, r, sg, nu))

    g = golden("reftest")
    for test, k, a in rt.all_inputs():
        for key, op, reg in rt.SECTIONS:
            want = g[f"{test}_r{k}_{key}"]
            got = rt.run_section(_Oracle, op, reg, a)
            if TOL == 0 and op != "p2d_visc":
                np.testing.assert_array_equal(got, want, err_msg=f"{test} r{k} {key}")
            else:
                e = rt.per_element_rel(got, want)
                assert np.nanmax(e, initial=0.0) <= rt.REL_ACC, (test, k, key)


def test_host_path_reference_comparison_sections(host):
    """The same sections through this library's host path (no accelerator
    enabled), per element against the reference's CPU result."""
    import reftest_inputs as rt
    g = golden("reftest")
    for test, k, a in rt.all_inputs()[::3]:
        for key, op, reg in rt.SECTIONS:
            e = rt.per_element_rel(rt.run_section(host, op, reg, a), g[f"{test}_r{k}_{key}"])
            assert np.nanmax(e, initial=0.0) <= rt.REL_ACC, (test, k, key, np.nanmax(e))


def test_oracle_vs_reference_library(built):
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference library not built here (sources absent)")
    ref.initialise()
    p = workloads.vortex_ring(1537, seed=99)
    mes = workloads.uniform_cube(257, seed=98)["coord"]
    for reg in REGS:
        _same(oracle.p3d_vel(p, mes, reg, 0.05), ref.p3d_vel(p, mes, reg, 0.05), TOL)
        _same(oracle.p3d_dvort(p, p, reg, 0.05), ref.p3d_dvort(p, p, reg, 0.05, same=True), TOL)


# ---- FP64 exact oracle -----------------------------------------------------
def test_exact_gaussian_series_matches_closed_form():
    rho = np.linspace(0.3, 0.7, 41)
    x = rho * rho
    G_s, K_s = exact._gauss_series_G(x), exact._gauss_series_K(x)
    from scipy.special import erf
    g = erf(rho / math.sqrt(2)) - rho * exact.SQ2PI * np.exp(-0.5 * x)
    G_c = g / rho ** 3
    K_c = (3 * G_c - exact.SQ2PI * np.exp(-0.5 * x)) / x
    np.testing.assert_allclose(G_s, G_c, rtol=1e-12)
    np.testing.assert_allclose(K_s, K_c, rtol=1e-9)
    assert math.isclose(exact._gauss_series_G(np.array([0.0]))[0], exact.SQ2PI / 3)
    assert math.isclose(exact._gauss_series_K(np.array([0.0]))[0], exact.SQ2PI / 5)


@pytest.mark.parametrize("reg", REGS)
def test_exact_close_to_reference_where_reference_is_accurate(built, reg):
    g = golden("p3d_cube")
    p, mes, s = g["particles"], g["mes"], float(g["sigma"])
    v, d = exact.p3d_vel_dvort(p, mes, None, reg, s, want_dvort=False)
    assert exact.rel_l2(g[f"velmes_{reg}"], v) < 5e-6
    _, d = exact.p3d_vel_dvort(p, p["coord"], p["vorticity"], reg, s, want_vel=False)
    assert exact.rel_l2(g[f"dvort_{reg}"], d) < (2e-4 if reg == "gaussian" else 5e-6)
    vi = exact.p3d_visc(p, p, reg, s, float(g["nu"]))
    if reg in ("winckelmans", "gaussian"):
        assert exact.rel_l2(g[f"visc_{reg}"], vi) < 5e-6


def test_exact_p2d_f3d_close_to_reference(built):
    g = golden("p2d_patch")
    q = g["particles"]
    for reg in REGS:
        assert exact.rel_l2(g[f"vel_{reg}"], exact.p2d_vel(q, q["coord"], reg, 0.05)) < 5e-6
    for reg in ("winckelmans", "gaussian"):
        assert exact.rel_l2(g[f"visc_{reg}"], exact.p2d_visc(q, q, reg, 0.05, 1e-3)) < 5e-6
    f = golden("f3d_sheet")
    assert exact.rel_l2(f["vel"], exact.f3d_vel(f["filaments"], f["mes"])) < 5e-6
    assert exact.rel_l2(f["dvort"], exact.f3d_dvort(f["filaments"], f["particles"])) < 5e-6


def test_compiled_exact_matches_numpy_exact(built):
    """The compiled FP64 oracle (the benchmark's error reports) against the
    numpy FP64 oracle, op by op; the vorticity field against the reference's
    formulation on its golden fixture."""
    g = golden("p3d_cube")
    p, mes, s, nu = g["particles"], g["mes"], float(g["sigma"]), float(g["nu"])
    for reg in REGS:
        np.testing.assert_allclose(oracle.exact_p3d_visc(p, p, reg, s, nu),
                                   exact.p3d_visc(p, p, reg, s, nu), rtol=1e-11, atol=1e-14)
        vort = oracle.exact_p3d_vort(p, mes, reg, s)
        if reg == "singular":
            assert not np.any(vort)
        else:
            assert exact.rel_l2(g[f"vort_{reg}"], vort) < 5e-6
    q = golden("p2d_patch")["particles"]
    for reg in REGS:
        np.testing.assert_allclose(oracle.exact_p2d_vel(q, q["coord"], reg, 0.05),
                                   exact.p2d_vel(q, q["coord"], reg, 0.05), rtol=1e-11, atol=1e-12)
        np.testing.assert_allclose(oracle.exact_p2d_visc(q, q, reg, 0.05, 1e-3),
                                   exact.p2d_visc(q, q, reg, 0.05, 1e-3), rtol=1e-11, atol=1e-14)
    f = golden("f3d_sheet")
    fil = f["filaments"]
    np.testing.assert_allclose(oracle.exact_f3d_vel(fil, f["mes"]), exact.f3d_vel(fil, f["mes"]),
                               rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(oracle.exact_f3d_dvort(fil, f["particles"]),
                               exact.f3d_dvort(fil, f["particles"]), rtol=1e-10, atol=1e-10)
    inf = oracle.exact_f3d_vel(fil[:200], f["mes"][:40], f["dirs"])
    assert exact.rel_l2(f["inf"], inf) < 5e-6
