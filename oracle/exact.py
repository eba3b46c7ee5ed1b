"""FP64 exact-math oracle -- TEST INFRASTRUCTURE ONLY.

The M2M interactions of cvortex evaluated in float64 with the exact error
function instead of the reference's Abramowitz & Stegun 7.1.26 approximation
(reference src/VortFunc.cpp:155-176). Formulas (reference file:line):

* P3D velocity (src/P3D.cpp:51-72, 230-251):
  u_t = -(1/4pi) sum_s g(rho)/r^3 (d x alpha_s), d = x_t - x_s, rho = r/|sigma|
* P3D stretching (src/P3D.cpp:86-114):
  (1/(4 pi sigma^3)) sum_s [G co - (3G - zeta)/r^2 (d.co) d],
  co = alpha_t x alpha_s, G = g/rho^3
* P3D viscous exchange (src/P3D.cpp:116-144):
  (2 nu/sigma^2) sum_s (alpha_s V_t - alpha_t V_s) eta(rho)
* P2D velocity and viscous exchange (src/P2D.cpp:49-69, 167-194)
* F3D velocity and stretching (src/F3D.cpp:34-85)
Coincident pairs contribute zero. G and (3G - zeta)/rho^2 use their Taylor
series below rho = 0.5 for the Gaussian, where the closed forms cancel.
Work is blocked over targets to bound memory.
"""
from __future__ import annotations

import math

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover - scipy is present on both hosts
    _erf = np.vectorize(math.erf)

SQ2PI = math.sqrt(2.0 / math.pi)
F64 = np.float64


def _gauss_series_G(x):
    # sqrt(2/pi) sum_n (-1)^n x^n / (2^n n! (2n+3)), x = rho^2
    out = np.zeros_like(x)
    for n in range(0, 16):
        c = ((-1) ** n) / (2.0 ** n * math.factorial(n) * (2 * n + 3))
        out += c * x ** n
    return SQ2PI * out


def _gauss_series_K(x):
    # (3G - zeta)/x = sqrt(2/pi) sum_{n>=1} (-1)^(n+1) 2n x^(n-1) / (2^n n! (2n+3))
    out = np.zeros_like(x)
    for n in range(1, 17):
        c = ((-1) ** (n + 1)) * 2.0 * n / (2.0 ** n * math.factorial(n) * (2 * n + 3))
        out += c * x ** (n - 1)
    return SQ2PI * out


def G_K(rho, reg):
    """G = g/rho^3 and K = (3G - zeta)/rho^2 for the 3D regularisations."""
    rho = np.asarray(rho, F64)
    x = rho * rho
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        if reg == "singular":
            G = 1.0 / (x * rho)
            K = 3.0 * G / x
        elif reg == "winckelmans":
            q = x + 1.0
            G = (q + 1.5) * q ** -2.5
            K = (3.0 * q + 7.5) * q ** -3.5
        elif reg == "planetary":
            inside = rho < 1.0
            G = np.where(inside, 1.0, 1.0 / (x * rho))
            K = np.where(inside, 0.0, 3.0 / (x * x * rho))
        elif reg == "gaussian":
            small = rho < 0.5
            g = _erf(rho / math.sqrt(2.0)) - rho * SQ2PI * np.exp(-0.5 * x)
            Gc = g / (x * rho)
            zeta = SQ2PI * np.exp(-0.5 * x)
            Kc = (3.0 * Gc - zeta) / x
            G = np.where(small, _gauss_series_G(x), Gc)
            K = np.where(small, _gauss_series_K(x), Kc)
        else:
            raise ValueError(reg)
    return G, K


def eta3(rho, reg):
    x = np.asarray(rho, F64) ** 2
    if reg == "winckelmans":
        return 52.5 * (x + 1.0) ** -4.5
    if reg == "gaussian":
        return SQ2PI * np.exp(-0.5 * x)
    return np.zeros_like(x)


def g2_over_r2(r2, sigma, reg):
    """g_2D(rho)/r^2."""
    s2 = float(sigma) ** 2
    x = r2 / s2
    with np.errstate(divide="ignore", invalid="ignore"):
        if reg == "singular":
            return 1.0 / r2
        if reg == "winckelmans":
            return (x + 2.0) / ((x + 1.0) ** 2 * s2)
        if reg == "planetary":
            return np.where(x < 1.0, 1.0 / s2, 1.0 / r2)
        if reg == "gaussian":
            return -np.expm1(-0.5 * x) / r2
    raise ValueError(reg)


def eta2(rho, reg):
    x = np.asarray(rho, F64) ** 2
    if reg == "winckelmans":
        a = x + 1.0
        return 24.0 * np.exp(4.0 / a ** 3) / a ** 4
    if reg == "gaussian":
        return np.exp(-0.5 * x)
    return np.zeros_like(x)


def _blocks(m, n, budget=4_000_000):
    b = max(1, budget // max(1, n))
    for i in range(0, m, b):
        yield slice(i, min(m, i + b))


def p3d_vel_dvort(src, tgt_pos, tgt_vort, reg, sigma, want_vel=True, want_dvort=True):
    """Velocity and/or stretching at targets (float64 arrays (M, 3))."""
    xs = src["coord"].astype(F64)
    a_s = src["vorticity"].astype(F64)
    xt = np.asarray(tgt_pos, F64)
    at = None if tgt_vort is None else np.asarray(tgt_vort, F64)
    m = xt.shape[0]
    vel = np.zeros((m, 3)) if want_vel else None
    dv = np.zeros((m, 3)) if want_dvort else None
    s = float(sigma)
    for sl in _blocks(m, xs.shape[0]):
        d = xt[sl, None, :] - xs[None, :, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        nz = r2 > 0
        r = np.sqrt(r2)
        G, K = G_K(r / abs(s), reg)
        G = np.where(nz, G, 0.0)
        K = np.where(nz, K, 0.0)
        c = np.cross(d, a_s[None, :, :])
        if want_vel:
            # g/r^3 = G/|sigma|^3
            vel[sl] = -np.einsum("ij,ijk->ik", G, c) / (4 * math.pi * abs(s) ** 3)
        if want_dvort:
            co = np.cross(at[sl, None, :], a_s[None, :, :])
            dco = np.einsum("ijk,ijk->ij", d, co)
            # (3G - zeta)/r^2 = K / sigma^2
            term = np.einsum("ij,ijk->ik", G, co) - np.einsum("ij,ijk->ik", K * dco / s ** 2, d)
            dv[sl] = term / (4 * math.pi * s ** 3)
    return vel, dv


def p3d_visc(src, tgt, reg, sigma, nu):
    xs = src["coord"].astype(F64)
    a_s = src["vorticity"].astype(F64)
    vs = src["volume"].astype(F64)
    xt = tgt["coord"].astype(F64)
    at = tgt["vorticity"].astype(F64)
    vt = tgt["volume"].astype(F64)
    m = xt.shape[0]
    out = np.zeros((m, 3))
    s = float(sigma)
    for sl in _blocks(m, xs.shape[0]):
        d = xs[None, :, :] - xt[sl, None, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        e = np.where(r2 > 0, eta3(np.sqrt(r2) / abs(s), reg), 0.0)
        w_s = np.einsum("ij,jk->ik", e, a_s) * vt[sl, None]
        w_t = at[sl] * (e @ vs)[:, None]
        out[sl] = (w_s - w_t) * (2.0 * nu / s ** 2)
    return out


def p2d_vel(src, mes, reg, sigma):
    xs = src["coord"].astype(F64)
    gs = src["vorticity"].astype(F64)
    xm = np.asarray(mes, F64)
    m = xm.shape[0]
    out = np.zeros((m, 2))
    for sl in _blocks(m, xs.shape[0]):
        d = xm[sl, None, :] - xs[None, :, :]
        r2 = d[..., 0] ** 2 + d[..., 1] ** 2
        h = np.where(r2 > 0, g2_over_r2(np.where(r2 > 0, r2, 1.0), sigma, reg), 0.0) * gs[None, :]
        out[sl, 0] = np.sum(h * d[..., 1], axis=1)
        out[sl, 1] = -np.sum(h * d[..., 0], axis=1)
    return out / (2 * math.pi)


def p2d_visc(src, tgt, reg, sigma, nu):
    xs = src["coord"].astype(F64)
    gs = src["vorticity"].astype(F64)
    As = src["area"].astype(F64)
    xt = tgt["coord"].astype(F64)
    gt = tgt["vorticity"].astype(F64)
    At = tgt["area"].astype(F64)
    m = xt.shape[0]
    out = np.zeros(m)
    s = float(sigma)
    for sl in _blocks(m, xs.shape[0]):
        d = xs[None, :, :] - xt[sl, None, :]
        r2 = d[..., 0] ** 2 + d[..., 1] ** 2
        e = np.where(r2 > 0, eta2(np.sqrt(r2) / abs(s), reg), 0.0)
        out[sl] = (e @ gs) * At[sl] - gt[sl] * (e @ As)
    return out * (2.0 * nu / s ** 2)


def f3d_vel(fil, mes):
    a = fil["start"].astype(F64)
    b = fil["end"].astype(F64)
    g = fil["strength"].astype(F64)
    xm = np.asarray(mes, F64)
    m = xm.shape[0]
    out = np.zeros((m, 3))
    with np.errstate(divide="ignore", invalid="ignore"):
        for sl in _blocks(m, a.shape[0]):
            r1 = xm[sl, None, :] - a[None]
            r2 = xm[sl, None, :] - b[None]
            r0 = r1 - r2
            c = np.cross(r1, r2)
            cc = np.einsum("ijk,ijk->ij", c, c)
            t1 = g[None, :] / (4 * math.pi * cc)
            t2 = (np.einsum("ijk,ijk->ij", r1, r0) / np.linalg.norm(r1, axis=-1)
                  - np.einsum("ijk,ijk->ij", r2, r0) / np.linalg.norm(r2, axis=-1))
            f = t1 * t2
            f = np.where(np.isfinite(f), f, 0.0)
            out[sl] = np.einsum("ij,ijk->ik", f, c)
    return out


def f3d_dvort(fil, ind):
    a = fil["start"].astype(F64)
    b = fil["end"].astype(F64)
    g = fil["strength"].astype(F64)
    xp = ind["coord"].astype(F64)
    wp = ind["vorticity"].astype(F64)
    m = xp.shape[0]
    out = np.zeros((m, 3))
    with np.errstate(divide="ignore", invalid="ignore"):
        for sl in _blocks(m, a.shape[0]):
            r1 = xp[sl, None, :] - a[None]
            r2 = xp[sl, None, :] - b[None]
            r0 = r1 - r2
            X = np.cross(r1, r0)
            X2 = np.einsum("ijk,ijk->ij", X, X)
            l1 = np.linalg.norm(r1, axis=-1)
            l2 = np.linalg.norm(r2, axis=-1)
            l0 = np.linalg.norm(r0, axis=-1)
            t1 = g[None, :] / (4 * math.pi)
            t212 = np.einsum("ijk,ijk->ij", r0, r1) / l1 - np.einsum("ijk,ijk->ij", r0, r2) / l2
            t222 = np.sqrt(X2) / l1 - np.sqrt(X2) / l2
            A = (-r0 / X2[..., None]) * (t1 * t212)[..., None]
            B = (3.0 / l0) * t1 * t222
            w = wp[sl, None, :]
            v = w * B[..., None] + np.cross(A, np.broadcast_to(w, A.shape))
            v = np.where(np.isfinite(v).all(axis=-1, keepdims=True), v, 0.0)
            out[sl] = v.sum(axis=1)
    return out


def term_magnitude(op, reg, sigma, nu, src, tgt=None, pts=None, co_bound=False):
    """Per target, the sum of the magnitudes of its terms, sum_s |term_s|
    (vector norms for vector outputs), with the same scaling as the op's
    result: the condition number of a target's sum is this over |result|.
    op: p3d_vel (src, pts), p3d_dvort (src, tgt), p3d_visc (src, tgt),
    p2d_vel (src, pts), p2d_visc (src, tgt), f3d_vel (fil=src, pts),
    f3d_dvort (fil=src, tgt).
    co_bound (p3d_dvort): bound each term's parts by |alpha_t| |alpha_s| in
    place of |alpha_t x alpha_s| (reference src/P3D.cpp:86-114 forms the
    cross product in FP32; for nearly parallel vorticities its rounding error
    is of order u |alpha_t| |alpha_s|, not u |alpha_t x alpha_s|)."""
    s = float(sigma)
    if op in ("p3d_vel", "p3d_dvort"):
        xs, a_s = src["coord"].astype(F64), src["vorticity"].astype(F64)
        xt = np.asarray(pts if op == "p3d_vel" else tgt["coord"], F64)
        d = xt[:, None, :] - xs[None, :, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        G, K = G_K(np.sqrt(r2) / abs(s), reg)
        G = np.where(r2 > 0, G, 0.0)
        K = np.where(r2 > 0, K, 0.0)
        if op == "p3d_vel":
            c = np.cross(d, a_s[None])
            return (np.abs(G) * np.linalg.norm(c, axis=-1)).sum(1) / (4 * math.pi * abs(s) ** 3)
        a_t = tgt["vorticity"].astype(F64)
        if co_bound:
            aa = np.linalg.norm(a_t, axis=1)[:, None] * np.linalg.norm(a_s, axis=1)[None]
            t = (np.abs(G) + np.abs(K) * r2 / s ** 2) * aa
            return t.sum(1) / (4 * math.pi * abs(s) ** 3)
        co = np.cross(a_t[:, None, :], a_s[None])
        dco = np.einsum("ijk,ijk->ij", d, co)
        t = G[..., None] * co - (K * dco / s ** 2)[..., None] * d
        return np.linalg.norm(t, axis=-1).sum(1) / (4 * math.pi * abs(s) ** 3)
    if op in ("p3d_visc", "p2d_visc"):
        two_d = op == "p2d_visc"
        xs, xt = src["coord"].astype(F64), tgt["coord"].astype(F64)
        d = xs[None] - xt[:, None]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        e = np.where(r2 > 0, (eta2 if two_d else eta3)(np.sqrt(r2) / abs(s), reg), 0.0)
        if two_d:
            w = (src["vorticity"].astype(F64)[None] * tgt["area"].astype(F64)[:, None]
                 - tgt["vorticity"].astype(F64)[:, None] * src["area"].astype(F64)[None])
            return np.abs(e * w).sum(1) * (2.0 * nu / s ** 2)
        w = (src["vorticity"].astype(F64)[None] * tgt["volume"].astype(F64)[:, None, None]
             - tgt["vorticity"].astype(F64)[:, None] * src["volume"].astype(F64)[None, :, None])
        return (np.abs(e) * np.linalg.norm(w, axis=-1)).sum(1) * (2.0 * nu / s ** 2)
    if op == "p2d_vel":
        xs, gs = src["coord"].astype(F64), src["vorticity"].astype(F64)
        d = np.asarray(pts, F64)[:, None] - xs[None]
        r2 = d[..., 0] ** 2 + d[..., 1] ** 2
        h = np.where(r2 > 0, g2_over_r2(np.where(r2 > 0, r2, 1.0), sigma, reg), 0.0) * gs[None]
        return (np.abs(h) * np.sqrt(r2)).sum(1) / (2 * math.pi)
    if op in ("f3d_vel", "f3d_dvort"):
        a, b = src["start"].astype(F64), src["end"].astype(F64)
        g = src["strength"].astype(F64)
        x = np.asarray(pts if op == "f3d_vel" else tgt["coord"], F64)
        with np.errstate(divide="ignore", invalid="ignore"):
            r1, r2 = x[:, None] - a[None], x[:, None] - b[None]
            r0 = r1 - r2
            l1, l2 = np.linalg.norm(r1, axis=-1), np.linalg.norm(r2, axis=-1)
            t212 = np.einsum("ijk,ijk->ij", r0, r1) / l1 - np.einsum("ijk,ijk->ij", r0, r2) / l2
            if op == "f3d_vel":
                c = np.cross(r1, r2)
                cc = np.einsum("ijk,ijk->ij", c, c)
                v = (g[None] / (4 * math.pi * cc) * t212)[..., None] * c
            else:
                X = np.cross(r1, r0)
                X2 = np.einsum("ijk,ijk->ij", X, X)
                t1 = g[None] / (4 * math.pi)
                A = (-r0 / X2[..., None]) * (t1 * t212)[..., None]
                B = (3.0 / np.linalg.norm(r0, axis=-1)) * t1 * (np.sqrt(X2) / l1 - np.sqrt(X2) / l2)
                w = np.broadcast_to(tgt["vorticity"].astype(F64)[:, None], A.shape)
                v = w * B[..., None] + np.cross(A, w)
            m = np.linalg.norm(v, axis=-1)
            return np.where(np.isfinite(m), m, 0.0).sum(1)
    raise ValueError(op)


def rel_l2(a, b):
    """||a - b||_2 / ||b||_2 over a whole output array."""
    a = np.asarray(a, F64).ravel()
    b = np.asarray(b, F64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def max_rel(a, b, floor=1e-30):
    """max_i |a_i - b_i| / max(|b_i|, floor) over target vectors (rows)."""
    a = np.asarray(a, F64)
    b = np.asarray(b, F64)
    if a.ndim == 1:
        a, b = a[:, None], b[:, None]
    num = np.linalg.norm(a - b, axis=1)
    den = np.maximum(np.linalg.norm(b, axis=1), floor)
    return float(np.max(num / den)) if len(num) else 0.0
