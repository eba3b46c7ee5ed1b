"""Inputs and sections of the reference's own CPU-vs-GPU comparison tests
(test infrastructure).

The reference ships two integration tests that run every M2M function once
on its accelerator and once on its CPU path and compare the two per element:
reference test/testsamecpugpuresultsingle.h:37-459 ("a single particle with
any vorticity") and test/testsamecpugpuresultmany.h:35-468 ("many particles
with vorticity"). Both draw their inputs from the LCG of
test/testmain.c:87-92 and run 10 repeats of 1,000 objects, sigma 0.3; the
single-object test runs first (test/testmain.c:101-102), so the many-object
test continues the same LCG stream. The bar is per element:
|a - b| / |a + b| <= 1e-5 wherever |a + b| > 2e-35
(testsamecpugpuresultmany.h:94-107).

This module regenerates those inputs bit for bit (float32 arithmetic as in
the C source) and lists every section with the call it makes.

One deviation: the P2D measurement points of both tests (p2mes,
mes_pts2d) are allocated but never written by the reference
(testsamecpugpuresultmany.h:59, testsamecpugpuresultsingle.h:66), so the
reference compares results at uninitialised points. Here the P2D sections
measure at the P2D particles' own coordinates, as the 3D sections do
(pmes[i] = particles[i].coord, testsamecpugpuresultmany.h:73).
"""
from __future__ import annotations

import numpy as np

from cvortex_gb300.abi import F3D_DTYPE, P2D_DTYPE, P3D_DTYPE

N_OBJ = 1000          # testsamecpugpuresult*.h: num_obj
REPEATS = 10          # max_repeats
SIGMA = 0.3           # reg_rad
NU = 0.1              # kinematic viscosity of the viscous sections
REL_ACC = 1e-5        # rel_acc
F32 = np.float32
_RAND_MAX = 2147483647
# (float)(RAND_MAX / max_float) with max_float = 10.f (int -> float, then a
# float division) and (float)(RAND_MAX / 0.01) (a double division)
_DIV10 = F32(F32(_RAND_MAX) / F32(10.0))
_DIV001 = F32(_RAND_MAX / 0.01)


class Mrand:
    """test/testmain.c:87-92: a static int state, x = x * 214013 + 2531011
    (in long, stored back into the int), result ((x >> 16) & 0x7fff) %
    RAND_MAX; the state starts at 0xF0F0F0F0."""

    def __init__(self):
        self.v = 0xF0F0F0F0 - (1 << 32)

    def __call__(self) -> int:
        v = (self.v * 214013 + 2531011) & 0xFFFFFFFF
        self.v = v - (1 << 32) if v & 0x80000000 else v
        return ((self.v >> 16) & 0x7FFF) % _RAND_MAX

    def f10(self):            # (float)mrand() / (float)(RAND_MAX / max_float)
        return F32(F32(self()) / _DIV10)

    def fvol(self):           # (float)mrand() / (float)(RAND_MAX / 0.01)
        return F32(F32(self()) / _DIV001)

    def fsym(self):           # ... - max_float / 2.f
        return F32(self.f10() - F32(5.0))


def _single_repeat(r: Mrand):
    """testsamecpugpuresultsingle.h:74-125 and :329-346."""
    n = N_OBJ
    p3 = np.zeros(n, P3D_DTYPE)
    t3 = np.zeros(n, P3D_DTYPE)
    p3["coord"][0] = [r.f10() for _ in range(3)]
    p3["vorticity"][0] = [r.fsym() for _ in range(3)]
    p3["volume"][0] = r.fvol()
    t3[0] = p3[0]
    for i in range(1, n):
        p3["coord"][i] = [r.f10() for _ in range(3)]
        p3["volume"][i] = r.fvol()
        t3[i] = p3[i]
        t3["vorticity"][i] = [r.fsym() for _ in range(3)]
    fil = np.zeros(n, F3D_DTYPE)
    fil["start"][0] = [r.f10() for _ in range(3)]
    fil["end"][0] = [r.f10() for _ in range(3)]
    fil["strength"][0] = r.fsym()
    for i in range(1, n):
        fil["start"][i] = [r.f10() for _ in range(3)]
        e = np.array([r.f10() for _ in range(3)], F32)
        # end = bsv_V3f_plus(end, bsv_V3f_mult(start, 0.01)), float arithmetic
        fil["end"][i] = e + fil["start"][i] * F32(0.01)
        fil["strength"][i] = 0.0
    p2 = np.zeros(n, P2D_DTYPE)
    t2 = np.zeros(n, P2D_DTYPE)
    p2["coord"][0] = [r.f10(), r.f10()]
    p2["vorticity"][0] = r.fsym()
    p2["area"][0] = r.fvol()
    t2[0] = p2[0]
    for i in range(1, n):
        p2["coord"][i] = [r.f10(), r.f10()]
        p2["area"][i] = r.fvol()
        t2[i] = p2[i]
        t2["vorticity"][i] = r.f10()
    return {"p3": p3, "t3": t3, "fil": fil, "p2": p2, "t2": t2}


def _many_repeat(r: Mrand):
    """testsamecpugpuresultmany.h:68-89 and :335-341."""
    n = N_OBJ
    p3 = np.zeros(n, P3D_DTYPE)
    for i in range(n):
        p3["coord"][i] = [r.f10() for _ in range(3)]
        p3["vorticity"][i] = [r.f10() for _ in range(3)]
        p3["volume"][i] = r.fvol()
    fil = np.zeros(n, F3D_DTYPE)
    for i in range(n):
        fil["start"][i] = [r.f10() for _ in range(3)]
        fil["end"][i] = [r.f10() for _ in range(3)]
        fil["strength"][i] = r.f10()
    p2 = np.zeros(n, P2D_DTYPE)
    for i in range(n):
        p2["coord"][i] = [r.f10(), r.f10()]
        p2["vorticity"][i] = r.f10()
        p2["area"][i] = r.fvol()
    return {"p3": p3, "t3": p3, "fil": fil, "p2": p2, "t2": p2}


def all_inputs():
    """[(test, repeat, arrays)] in the order the reference test program
    draws them: the single-object test's 10 repeats, then the many-object
    test's 10 repeats."""
    r = Mrand()
    out = [("single", k, _single_repeat(r)) for k in range(REPEATS)]
    out += [("many", k, _many_repeat(r)) for k in range(REPEATS)]
    return out


# Sections of both tests, in their order: (key, op, regularisation).
# P3D vel at the particles' coordinates; P3D dvort / visc of the target set
# t3 (the particles themselves in the many-object test); F3D vel at the
# particles' coordinates and F3D dvort of t3; P2D vel at the P2D particles'
# coordinates; P2D visc of t2.
SECTIONS = (
    [(f"p3d_vel_{g}", "p3d_vel", g) for g in ("singular", "planetary", "gaussian", "winckelmans")]
    + [(f"p3d_dvort_{g}", "p3d_dvort", g) for g in ("singular", "planetary", "gaussian", "winckelmans")]
    + [(f"p3d_visc_{g}", "p3d_visc", g) for g in ("gaussian", "winckelmans")]
    + [("f3d_vel", "f3d_vel", None), ("f3d_dvort", "f3d_dvort", None)]
    + [(f"p2d_vel_{g}", "p2d_vel", g) for g in ("singular", "planetary", "gaussian", "winckelmans")]
    + [(f"p2d_visc_{g}", "p2d_visc", g) for g in ("gaussian", "winckelmans")]
)


def run_section(cv, op, reg, a):
    """One section's call through the cvtx_ ABI of library `cv` (a
    cvortex_gb300.abi.Cvtx over this library or the reference's)."""
    if op == "p3d_vel":
        return cv.p3d_vel(a["p3"], a["p3"]["coord"], reg, SIGMA)
    if op == "p3d_dvort":
        return cv.p3d_dvort(a["p3"], a["t3"], reg, SIGMA, same=a["t3"] is a["p3"])
    if op == "p3d_visc":
        return cv.p3d_visc(a["p3"], a["t3"], reg, SIGMA, NU, same=a["t3"] is a["p3"])
    if op == "f3d_vel":
        return cv.f3d_vel(a["fil"], a["p3"]["coord"])
    if op == "f3d_dvort":
        return cv.f3d_dvort(a["fil"], a["t3"])
    if op == "p2d_vel":
        return cv.p2d_vel(a["p2"], a["p2"]["coord"], reg, SIGMA)
    if op == "p2d_visc":
        return cv.p2d_visc(a["p2"], a["t2"], reg, SIGMA, NU, same=a["t2"] is a["p2"])
    raise ValueError(op)


def per_element_rel(a, b):
    """|a - b| / |a + b| per output element (vector norms for vector
    outputs), NaN where |a + b| <= 2e-35 (the reference skips those)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    if a.ndim == 1:
        a, b = a[:, None], b[:, None]
    dm = np.sqrt(((a - b).astype(np.float64) ** 2).sum(axis=1))
    dp = np.sqrt(((a + b).astype(np.float64) ** 2).sum(axis=1))
    out = np.full(len(a), np.nan)
    ok = dp > 2e-35
    out[ok] = dm[ok] / dp[ok]
    return out
