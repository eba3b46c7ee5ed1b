"""Oracle (test infrastructure): numpy restatement of the reference's particle
redistribution, cvtx_P3D_redistribute_on_grid / cvtx_P2D_redistribute_on_grid
(reference src/P3D.cpp:508-634, src/P2D.cpp:283-404, helpers in
src/redistribution_helper_funcs.cpp:34-112, src/array_methods.cpp:150-194,
redistribution functions src/RedistFunc.cpp:35-96, grid keys
src/UIntKey96.cpp:49-141, octree order src/GridParticleOcttree.cpp:139-190).

Pinned against the reference library itself (built by oracle/build_ref.sh
through the reference's complete MSVC branch of matching_leading_bits, whose
GCC branch is a stub, src/UIntKey96.h:240-265) on the golden fixture
tests/golden/redist.npz: same counts, coordinates and order bit for bit;
strengths to 2^-21 of the largest, because grid-point sums are taken here in
FP64 in particle order and the reference sums in FP32 per OpenMP thread.

Test infrastructure: only tests/ use it, to check the library's results.
"""
from __future__ import annotations

import math

import numpy as np

F32 = np.float32
RADIUS = {"lambda0": 0.5, "lambda1": 1.0, "lambda2": 1.5, "lambda3": 2.0, "m4p": 2.0}


def redist_func(name: str, u):
    """The reference redistribution functions, FP32, one rounding per op in
    the order of the C expressions (src/RedistFunc.cpp:35-96)."""
    u = np.asarray(u, F32)
    one, two, three, half = F32(1), F32(2), F32(3), F32(0.5)
    if name == "lambda0":
        return np.where(u < half, one, F32(0))
    if name == "lambda1":
        return np.where(u <= one, one - u, F32(0))
    if name == "lambda2":
        a = one - u * u
        b = (half * (one - u)) * (two - u)
        return np.where(u < half, a, np.where(u < F32(1.5), b, F32(0)))
    if name == "lambda3":
        a = (half * (one - u * u)) * (two - u)
        b = ((F32(1.0 / 6.0) * (one - u)) * (two - u)) * (three - u)
        return np.where(u < one, a, np.where(u < two, b, F32(0)))
    if name == "m4p":
        a = (one - (F32(2.5) * u) * u) + ((F32(1.5) * u) * u) * u
        b = ((half * (one - u)) * (two - u)) * (two - u)
        return np.where(u < one, a, np.where(u < two, b, F32(0)))
    raise ValueError(name)


def _roundf(x):
    """C roundf (half away from zero) of FP32 values, exact: x +- 0.5 is
    exact in FP64 for every FP32 x."""
    x = np.asarray(x, F32).astype(np.float64)
    return np.where(x >= 0, np.floor(x + 0.5), np.ceil(x - 0.5)).astype(F32)


def _morton(keys: np.ndarray) -> np.ndarray:
    """Interleave bits: axis d of bit b -> bit dims*b + d."""
    dims = keys.shape[1]
    code = np.zeros(len(keys), np.uint64)
    for b in range(32 if dims == 2 else 21):
        for d in range(dims):
            code |= ((keys[:, d].astype(np.uint64) >> np.uint64(b)) & np.uint64(1)) << \
                np.uint64(dims * b + d)
    return code


def _grid(pos: np.ndarray, fname: str, gd: float):
    gd = F32(gd)
    radius = int(math.floor(RADIUS[fname] + 0.5))
    mn = pos.min(axis=0).astype(F32)
    mean = (pos.astype(np.float64).sum(axis=0) / len(pos)).astype(F32)
    lo = mn - F32(radius) * gd
    dc = _roundf((mean - lo) / gd) + F32(5)
    return mean - dc * gd, gd, F32(1) / gd, radius


def cells(pos: np.ndarray, strength: np.ndarray, fname: str, gd: float):
    """(grid keys, summed strengths, corner) in ascending Morton order."""
    pos = np.ascontiguousarray(pos, F32)
    dims = pos.shape[1]
    strength = np.asarray(strength, F32).reshape(len(pos), -1)
    mn, gd32, rgd, radius = _grid(pos, fname, gd)
    base = _roundf((pos - mn) * rgd).astype(np.int64)
    w = 2 * radius + 1
    offs = np.array(np.meshgrid(*([np.arange(-radius, radius + 1)] * dims), indexing="ij"))
    offs = offs.reshape(dims, -1).T                           # stencil, x outermost
    keys = base[:, None, :] + offs[None, :, :]                # particle, stencil, dim
    npos = mn + gd32 * keys.astype(F32)
    u = np.abs((pos[:, None, :] - npos) * rgd)
    frac = redist_func(fname, u[..., 0])
    for d in range(1, dims):
        frac = frac * redist_func(fname, u[..., d])
    contrib = strength[:, None, :] * frac[..., None]          # particle, stencil, comp
    keys = keys.reshape(-1, dims)
    contrib = contrib.reshape(-1, contrib.shape[-1])
    keep = np.any(contrib != 0, axis=1)
    keys, contrib = keys[keep], contrib[keep]
    code = _morton(keys)
    uniq, first, inv = np.unique(code, return_index=True, return_inverse=True)
    acc = np.zeros((len(uniq), contrib.shape[1]))
    np.add.at(acc, inv, contrib.astype(np.float64))           # in particle order
    return keys[first].astype(np.int64), acc.astype(F32), mn


def _strength_threshold(strs: np.ndarray, n_desired: int) -> float:
    """src/redistribution_helper_funcs.cpp:34-85."""
    n = len(strs)
    minv, maxv = float(strs.min()), float(strs.max())
    if n < n_desired:
        return float(F32(maxv * 1.05))
    ng, tol, k = 1024, 0.01, 0
    while True:
        rng = (maxv - minv) * 1.05
        guess = np.array([F32(minv + i * rng / float(F32(ng - 1))) for i in range(ng)], F32)
        b = np.floor((ng - 1) * (strs.astype(np.float64) - minv) / rng).astype(np.int64)
        cnt = np.bincount(np.clip(b, 0, ng - 1), minlength=ng).astype(np.int64)
        acc = int(cnt[ng - 1])
        for i in range(ng - 2, -1, -1):
            maxv, minv = float(guess[i + 1]), float(guess[i])
            acc += int(cnt[i])
            cnt[i] = acc
            if acc > n_desired:
                k = i + 1
                break
        if (minv == maxv or k < 1 or cnt[k] == cnt[k - 1] or
                abs(float(F32(F32(n_desired - cnt[k]) / F32(n_desired)))) < float(F32(tol)) * 0.6):
            break
    return float(guess[k])


def _remove(vort: np.ndarray, strs: np.ndarray, thr: float, max_keep: int):
    keep = (strs > F32(thr)) & (np.arange(len(strs)) < max_keep)
    deficit = np.zeros(vort.shape[1], F32)
    for v in vort[~keep]:
        deficit = v + deficit
    n = int(keep.sum())
    with np.errstate(divide="ignore", invalid="ignore"):
        deficit = deficit / F32(n)
    return keep, vort[keep] + deficit


def redistribute(pos, strength, fname: str, gd: float, negligible: float, max_out: int | None):
    """Full redistribution: returns (count, coords, strengths) -- coords and
    strengths of the particles written to the output (None if max_out is
    None, i.e. a NULL output array)."""
    pos = np.asarray(pos, F32)
    if len(pos) == 0:
        return 0, None, None
    keys, vort, mn = cells(pos, strength, fname, gd)
    gd32 = F32(gd)
    coord = mn + gd32 * keys.astype(F32)
    if vort.shape[1] == 3:
        norm = lambda v: np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])
    else:
        norm = lambda v: np.abs(v[:, 0])
    strs = norm(vort)
    mean = F32(F32(strs.astype(np.float64).sum()) / F32(len(strs))) if len(strs) else F32(0)
    keep, vort = _remove(vort, strs, float(mean * F32(negligible)), len(strs))
    coord = coord[keep]
    strs = norm(vort)
    if max_out is None:
        return len(vort), None, None
    if len(vort) > max_out:
        thr = _strength_threshold(strs, max_out)
        keep, vort = _remove(vort, strs, thr, max_out)
        coord = coord[keep]
    return len(vort), coord, vort
