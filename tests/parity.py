"""Parity assertions shared by the GPU tests.

Bar: relative L2 error <= 1e-5 per output array against the reference path.

Gaussian regularisation: below rho_c the kernels evaluate g/rho^3 and
(3 g/rho^3 - zeta)/rho^2 from their exact series, where the reference's erf
approximation cancels (reference src/VortFunc.cpp:164-174). For that
regularisation parity is asserted on targets with no source closer than
rho_c * |sigma|, and, when an FP64 result is given, the GPU's error against
FP64 on all targets must not exceed the reference's own.
"""
import numpy as np

import oracle
from oracle import exact

TOL = 1e-5


def min_rho(src_xyz, tgt_xyz, sigma):
    """Smallest nonzero separation / |sigma| from each target to the sources."""
    if len(src_xyz) > 50_000:
        return min_rho_tree(src_xyz, tgt_xyz, sigma)
    s = np.asarray(src_xyz, np.float64)
    out = np.empty(len(tgt_xyz))
    for i, t in enumerate(np.asarray(tgt_xyz, np.float64)):
        r2 = ((s - t) ** 2).sum(axis=1)
        r2 = r2[r2 > 0]
        out[i] = np.sqrt(r2.min()) / abs(sigma) if len(r2) else np.inf
    return out


def min_rho_tree(src_xyz, tgt_xyz, sigma, k=8):
    """min_rho through a k-d tree (large source sets): the nearest of the k
    nearest sources at a nonzero distance."""
    from scipy.spatial import cKDTree
    s = np.asarray(src_xyz, np.float64)
    t = np.asarray(tgt_xyz, np.float64)
    d, _ = cKDTree(s).query(t, k=min(k, len(s)))
    d = np.where(d > 0, d, np.inf)
    return d.min(axis=1) / abs(sigma)


def check(got, want, reg=None, tgt_xyz=None, src_xyz=None, sigma=None, fp64=None, tol=TOL,
          rho_c=0.5):
    got = np.asarray(got)
    assert np.all(np.isfinite(got)), "non-finite output"
    if reg != "gaussian" or tgt_xyz is None:
        e = exact.rel_l2(got, want)
        assert e <= tol, f"rel L2 vs reference {e:.3e}"
        return
    keep = min_rho(src_xyz, tgt_xyz, sigma) >= rho_c
    if keep.any():
        e = exact.rel_l2(got[keep], np.asarray(want)[keep])
        assert e <= tol, f"rel L2 vs reference on {keep.sum()} unaffected targets {e:.3e}"
    if fp64 is not None:
        e_gpu, e_ref = exact.rel_l2(got, fp64), exact.rel_l2(want, fp64)
        assert e_gpu <= max(e_ref, 1e-6) * 1.05, f"vs FP64: gpu {e_gpu:.3e}, reference {e_ref:.3e}"


def same_up_to_rounding(p, reg, name, got, base, what, sigma):
    """Two FP32 evaluations of the same P3D velocity or stretching sums
    (`name` "vel" or "dvort"; particles `p` acting on themselves): equal
    within 1e-5 relative on every target except targets whose sums cancel
    (one per hundred at most; the singular stretching of a ring has 0.3 %).
    The 32 worst of those must lie within the FP32 bound 8 u sum_s |term_s|
    of the FP64 value in both evaluations. A fault confined to one packed
    lane or one target slot would show on a fixed fraction (1/2 .. 1/6) of
    all targets."""
    n = len(base)
    assert np.all(np.isfinite(got)), what
    err = np.linalg.norm(got - base, axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(base, axis=1),
                                  np.sqrt(np.mean(np.sum(base ** 2, axis=1)))), 1e-30)
    rel = err / scale
    bad = np.flatnonzero(rel > 1e-5)
    assert len(bad) <= max(n // 100, 1), (what, len(bad))
    if len(bad) == 0:
        return
    worst = bad[np.argsort(rel[bad])[-32:]]
    sub = p[worst].copy()
    ev, ed = oracle.exact_p3d_vel_dvort(p, sub["coord"], sub["vorticity"], reg, sigma,
                                        want_vel=name == "vel", want_dvort=name == "dvort")
    ex = ev if name == "vel" else ed
    # the pair terms' own FP32 rounding (the stretching's alpha_t x alpha_s)
    # counts at its parts' magnitude
    mag = exact.term_magnitude("p3d_" + name, reg, sigma, 0.0, p, tgt=sub, pts=sub["coord"],
                               co_bound=True)
    bound = np.maximum(1e-5 * np.linalg.norm(ex, axis=1), 8 * 2.0 ** -24 * mag)
    for arr in (got, base):
        e = np.linalg.norm(arr[worst].astype(np.float64) - ex, axis=1)
        assert np.all(e <= bound), (what, worst[e > bound], e[e > bound], bound[e > bound])
