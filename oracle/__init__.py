"""The oracle -- TEST INFRASTRUCTURE ONLY.

Three checkers for the GB300 library, none of which the product imports:

* ``lib()``: ``cvtx_oracle.c``, a plain-C restatement of the reference
  cvortex CPU (OpenMP) path for the M2M interactions, built here by ``build()``
  into ``oracle/lib/libcvtx_oracle.so``. It runs anywhere gcc runs (x86-64 or
  aarch64), so tests, the smoke check and the CPU-baseline leg of the
  benchmark can use it where the reference sources are absent.
* ``ref_lib()``: the reference library itself, compiled from the reference
  sources by ``oracle/build_ref.sh`` into ``oracle/_ref/libcvtx_ref.so`` when
  those sources are present. It pins the restatement (tests compare the two)
  and generates the golden fixtures under ``tests/golden``.
* ``oracle.exact``: the same formulas in float64 with the exact error
  function, i.e. the "error vs FP64" reference (independent of the reference
  implementation and of FP32 rounding); ``exact_p3d_vel_dvort`` is the same
  in compiled C for large samples, as are the ``exact_*`` functions of this
  module for the other ops.
* ``oracle.redist``: a numpy restatement of the reference's particle
  redistribution, pinned to the reference library's outputs (golden
  fixture ``tests/golden/redist.npz``; see that module).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
LIB = HERE / "lib" / "libcvtx_oracle.so"
REF_LIB = HERE / "_ref" / "libcvtx_ref.so"
# The reference checkout: $CVTX_REFERENCE_ROOT, else a directory named
# "reference" beside this repository's root; absent on hosts without it.
REFERENCE_ROOT = Path(os.environ.get("CVTX_REFERENCE_ROOT") or (REPO.parent / "reference"))


def build(force: bool = False) -> Path:
    """Compile the C restatement with OpenMP (gcc, -O2, no fast-math)."""
    src = HERE / "cvtx_oracle.c"
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11",
               "-I", str(REPO / "include"), str(src), "-o", str(LIB), "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


def build_ref() -> Path | None:
    """Compile the reference CPU library if its sources are present."""
    if not (REFERENCE_ROOT / "src").is_dir():
        return None
    subprocess.run(["bash", str(HERE / "build_ref.sh"), str(REFERENCE_ROOT)], check=True,
                   capture_output=True)
    return REF_LIB if REF_LIB.exists() else None


_vp, _i, _f = C.c_void_p, C.c_int, C.c_float
_SIGS = {
    "oracle_regfunc": (_f, [_i, _i, _f]),
    "oracle_P3D_M2M_vel": (None, [_vp, _i, _vp, _i, _vp, _i, _f]),
    "oracle_P3D_M2M_dvort": (None, [_vp, _i, _vp, _i, _vp, _i, _f]),
    "oracle_P3D_M2M_visc_dvort": (None, [_vp, _i, _vp, _i, _vp, _i, _f, _f]),
    "oracle_P3D_M2M_vort": (None, [_vp, _i, _vp, _i, _vp, _i, _f]),
    "oracle_P2D_M2M_vel": (None, [_vp, _i, _vp, _i, _vp, _i, _f]),
    "oracle_P2D_M2M_visc_dvort": (None, [_vp, _i, _vp, _i, _vp, _i, _f, _f]),
    "oracle_F3D_M2M_vel": (None, [_vp, _i, _vp, _i, _vp]),
    "oracle_F3D_M2M_dvort": (None, [_vp, _i, _vp, _i, _vp]),
    "oracle_F3D_inf_mtrx": (None, [_vp, _i, _vp, _vp, _i, _vp]),
    "oracle_num_threads": (_i, []),
    "oracle_exact_P3D_vel_dvort": (None, [_vp, _vp, _i, _vp, _vp, _i, _i, C.c_double, _vp, _vp]),
    "oracle_exact_P3D_visc": (None, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _i, C.c_double,
                                     C.c_double, _vp]),
    "oracle_exact_P3D_vort": (None, [_vp, _vp, _i, _vp, _i, _i, C.c_double, _vp]),
    "oracle_exact_P2D_vel": (None, [_vp, _vp, _i, _vp, _i, _i, C.c_double, _vp]),
    "oracle_exact_P2D_visc": (None, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _i, C.c_double,
                                     C.c_double, _vp]),
    "oracle_exact_F3D_vel": (None, [_vp, _vp, _vp, _i, _vp, _vp, _i, _vp]),
    "oracle_exact_F3D_dvort": (None, [_vp, _vp, _vp, _i, _vp, _vp, _i, _vp]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build()
        _lib = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(_lib, name)
            fn.restype, fn.argtypes = res, args
    return _lib


def ref_lib():
    """numpy front end (cvortex_gb300.abi.Cvtx) over the reference library
    (oracle/_ref), or None when it has not been built."""
    if not REF_LIB.exists():
        return None
    from cvortex_gb300.abi import Cvtx
    return Cvtx(REF_LIB, extensions=False)


REG = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}


def _ptrs(arr):
    from cvortex_gb300.abi import ptr_array
    return ptr_array(arr)


def _a(x):
    return x.ctypes.data


# ---- numpy wrappers of the C restatement -----------------------------------
def p3d_vel(src, mes, reg, sigma):
    p = _ptrs(src)
    mes = np.ascontiguousarray(mes, np.float32)
    out = np.zeros((mes.shape[0], 3), np.float32)
    lib().oracle_P3D_M2M_vel(_a(p), len(src), _a(mes), mes.shape[0], _a(out), REG[reg], sigma)
    return out


def p3d_dvort(src, ind, reg, sigma):
    p, q = _ptrs(src), _ptrs(ind)
    out = np.zeros((len(ind), 3), np.float32)
    lib().oracle_P3D_M2M_dvort(_a(p), len(src), _a(q), len(ind), _a(out), REG[reg], sigma)
    return out


def p3d_visc(src, ind, reg, sigma, nu):
    p, q = _ptrs(src), _ptrs(ind)
    out = np.zeros((len(ind), 3), np.float32)
    lib().oracle_P3D_M2M_visc_dvort(_a(p), len(src), _a(q), len(ind), _a(out), REG[reg], sigma, nu)
    return out


def p3d_vort(src, mes, reg, sigma):
    p = _ptrs(src)
    mes = np.ascontiguousarray(mes, np.float32)
    out = np.zeros((mes.shape[0], 3), np.float32)
    lib().oracle_P3D_M2M_vort(_a(p), len(src), _a(mes), mes.shape[0], _a(out), REG[reg], sigma)
    return out


def p2d_vel(src, mes, reg, sigma):
    p = _ptrs(src)
    mes = np.ascontiguousarray(mes, np.float32)
    out = np.zeros((mes.shape[0], 2), np.float32)
    lib().oracle_P2D_M2M_vel(_a(p), len(src), _a(mes), mes.shape[0], _a(out), REG[reg], sigma)
    return out


def p2d_visc(src, ind, reg, sigma, nu):
    p, q = _ptrs(src), _ptrs(ind)
    out = np.zeros(len(ind), np.float32)
    lib().oracle_P2D_M2M_visc_dvort(_a(p), len(src), _a(q), len(ind), _a(out), REG[reg], sigma, nu)
    return out


def f3d_vel(fil, mes):
    p = _ptrs(fil)
    mes = np.ascontiguousarray(mes, np.float32)
    out = np.zeros((mes.shape[0], 3), np.float32)
    lib().oracle_F3D_M2M_vel(_a(p), len(fil), _a(mes), mes.shape[0], _a(out))
    return out


def f3d_dvort(fil, ind):
    p, q = _ptrs(fil), _ptrs(ind)
    out = np.zeros((len(ind), 3), np.float32)
    lib().oracle_F3D_M2M_dvort(_a(p), len(fil), _a(q), len(ind), _a(out))
    return out


def f3d_inf_mtrx(fil, mes, dirs):
    p = _ptrs(fil)
    mes = np.ascontiguousarray(mes, np.float32)
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros((mes.shape[0], len(fil)), np.float32)
    lib().oracle_F3D_inf_mtrx(_a(p), len(fil), _a(mes), _a(dirs), mes.shape[0], _a(out))
    return out


def exact_p3d_vel_dvort(src, tgt_xyz, tgt_alpha, reg, sigma, want_vel=True, want_dvort=True):
    """FP64 exact-math velocity / stretching (compiled, OpenMP); see
    oracle_exact_P3D_vel_dvort in cvtx_oracle.c."""
    sx = np.ascontiguousarray(src["coord"], np.float64)
    sa = np.ascontiguousarray(src["vorticity"], np.float64)
    tx = np.ascontiguousarray(tgt_xyz, np.float64)
    ta = None if tgt_alpha is None else np.ascontiguousarray(tgt_alpha, np.float64)
    m = tx.shape[0]
    vel = np.zeros((m, 3)) if want_vel else None
    dv = np.zeros((m, 3)) if want_dvort else None
    lib().oracle_exact_P3D_vel_dvort(_a(sx), _a(sa), len(sx), _a(tx),
                                     None if ta is None else _a(ta), m, REG[reg], float(sigma),
                                     None if vel is None else _a(vel),
                                     None if dv is None else _a(dv))
    return vel, dv


def _d(x):
    return np.ascontiguousarray(x, np.float64)


def exact_p3d_visc(src, tgt, reg, sigma, nu):
    """FP64 exact-math P3D viscous exchange at the particles `tgt`."""
    sx, sa, sv = _d(src["coord"]), _d(src["vorticity"]), _d(src["volume"])
    tx, ta, tv = _d(tgt["coord"]), _d(tgt["vorticity"]), _d(tgt["volume"])
    out = np.zeros((len(tgt), 3))
    lib().oracle_exact_P3D_visc(_a(sx), _a(sa), _a(sv), len(src), _a(tx), _a(ta), _a(tv),
                                len(tgt), REG[reg], float(sigma), float(nu), _a(out))
    return out


def exact_p3d_vort(src, mes, reg, sigma):
    """FP64 exact-math P3D vorticity field (5 sigma box) at points `mes`."""
    sx, sa, tx = _d(src["coord"]), _d(src["vorticity"]), _d(mes)
    out = np.zeros((tx.shape[0], 3))
    lib().oracle_exact_P3D_vort(_a(sx), _a(sa), len(src), _a(tx), tx.shape[0], REG[reg],
                                float(sigma), _a(out))
    return out


def exact_p2d_vel(src, mes, reg, sigma):
    """FP64 exact-math P2D velocity at points `mes` (M, 2)."""
    sx, sg, tx = _d(src["coord"]), _d(src["vorticity"]), _d(mes)
    out = np.zeros((tx.shape[0], 2))
    lib().oracle_exact_P2D_vel(_a(sx), _a(sg), len(src), _a(tx), tx.shape[0], REG[reg],
                               float(sigma), _a(out))
    return out


def exact_p2d_visc(src, tgt, reg, sigma, nu):
    """FP64 exact-math P2D viscous exchange at the particles `tgt`."""
    sx, sg, sa = _d(src["coord"]), _d(src["vorticity"]), _d(src["area"])
    tx, tg, ta = _d(tgt["coord"]), _d(tgt["vorticity"]), _d(tgt["area"])
    out = np.zeros(len(tgt))
    lib().oracle_exact_P2D_visc(_a(sx), _a(sg), _a(sa), len(src), _a(tx), _a(tg), _a(ta),
                                len(tgt), REG[reg], float(sigma), float(nu), _a(out))
    return out


def exact_f3d_vel(fil, mes, dirs=None):
    """FP64 exact-math F3D velocity at points `mes`; with `dirs`, the
    influence matrix (rows: points, columns: filaments)."""
    fa, fb, fg, tx = _d(fil["start"]), _d(fil["end"]), _d(fil["strength"]), _d(mes)
    m = tx.shape[0]
    dd = None if dirs is None else _d(dirs)
    out = np.zeros((m, len(fil)) if dirs is not None else (m, 3))
    lib().oracle_exact_F3D_vel(_a(fa), _a(fb), _a(fg), len(fil), _a(tx),
                               None if dd is None else _a(dd), m, _a(out))
    return out


def exact_f3d_dvort(fil, ind):
    """FP64 exact-math F3D vortex stretching of the particles `ind`."""
    fa, fb, fg = _d(fil["start"]), _d(fil["end"]), _d(fil["strength"])
    tx, ta = _d(ind["coord"]), _d(ind["vorticity"])
    out = np.zeros((len(ind), 3))
    lib().oracle_exact_F3D_dvort(_a(fa), _a(fb), _a(fg), len(fil), _a(tx), _a(ta), len(ind),
                                 _a(out))
    return out


def regfunc(reg: str, which: str, rho: float) -> float:
    w = {"g3": 0, "g2": 1, "zeta3": 2, "eta3": 3, "eta2": 4}[which]
    return float(lib().oracle_regfunc(REG[reg], w, rho))
