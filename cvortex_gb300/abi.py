"""ctypes mirror of the cvtx_ C ABI served by libcvortex.so.

The raw entry points keep the reference's names and argument order
(include/cvortex/libcvtx.h of cvortex 0.3.8); ``Cvtx`` adds numpy
conveniences that build the pointer arrays the ABI takes, the way callers of
the reference do (reference bench/bencharraysetup.c:43-58: one particle array
plus an array of pointers into it).

The library is built in-tree by ``cvortex_gb300.build`` into
``cvortex_gb300/lib/libcvortex.so``; loading fails loudly if it is missing.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libcvortex.so"

# ---- record layouts (byte-compatible with the C structs) --------------------
P3D_DTYPE = np.dtype([("coord", "<f4", (3,)), ("vorticity", "<f4", (3,)), ("volume", "<f4")])
P2D_DTYPE = np.dtype([("coord", "<f4", (2,)), ("vorticity", "<f4"), ("area", "<f4")])
F3D_DTYPE = np.dtype([("start", "<f4", (3,)), ("end", "<f4", (3,)), ("strength", "<f4")])
assert P3D_DTYPE.itemsize == 28 and P2D_DTYPE.itemsize == 16 and F3D_DTYPE.itemsize == 28

REG_IDS = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}


class bsv_V3f(C.Structure):
    _fields_ = [("x", C.c_float * 3)]


class bsv_V2f(C.Structure):
    _fields_ = [("x", C.c_float * 2)]


class cvtx_P3D(C.Structure):
    _fields_ = [("coord", bsv_V3f), ("vorticity", bsv_V3f), ("volume", C.c_float)]


class cvtx_F3D(C.Structure):
    _fields_ = [("start", bsv_V3f), ("end", bsv_V3f), ("strength", C.c_float)]


class cvtx_P2D(C.Structure):
    _fields_ = [("coord", bsv_V2f), ("vorticity", C.c_float), ("area", C.c_float)]


FN_F_F = C.CFUNCTYPE(C.c_float, C.c_float)
FN_COMB = C.CFUNCTYPE(None, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float))


class cvtx_VortFunc(C.Structure):
    _fields_ = [("g_3D", FN_F_F), ("g_2D", FN_F_F), ("zeta_3D", FN_F_F),
                ("combined_3D", FN_COMB), ("eta_3D", FN_F_F), ("eta_2D", FN_F_F),
                ("cl_kernel_name_ext", C.c_char * 32)]


class cvtx_RedistFunc(C.Structure):
    _fields_ = [("func", FN_F_F), ("radius", C.c_float)]


_vp = C.c_void_p
_i = C.c_int
_f = C.c_float
_VF = C.POINTER(cvtx_VortFunc)

# name: (restype, argtypes). Pointer arrays and result arrays travel as void*.
_SIGS = {
    "cvtx_initialise": (None, []),
    "cvtx_finalise": (None, []),
    "cvtx_information": (C.c_char_p, []),
    "cvtx_num_accelerators": (_i, []),
    "cvtx_num_enabled_accelerators": (_i, []),
    "cvtx_accelerator_name": (C.c_char_p, [_i]),
    "cvtx_accelerator_enabled": (_i, [_i]),
    "cvtx_accelerator_enable": (None, [_i]),
    "cvtx_accelerator_disable": (None, [_i]),
    "cvtx_VortFunc_singular": (cvtx_VortFunc, []),
    "cvtx_VortFunc_winckelmans": (cvtx_VortFunc, []),
    "cvtx_VortFunc_planetary": (cvtx_VortFunc, []),
    "cvtx_VortFunc_gaussian": (cvtx_VortFunc, []),
    "cvtx_RedistFunc_lambda0": (cvtx_RedistFunc, []),
    "cvtx_RedistFunc_lambda1": (cvtx_RedistFunc, []),
    "cvtx_RedistFunc_lambda2": (cvtx_RedistFunc, []),
    "cvtx_RedistFunc_lambda3": (cvtx_RedistFunc, []),
    "cvtx_RedistFunc_m4p": (cvtx_RedistFunc, []),
    "cvtx_P3D_S2S_vel": (bsv_V3f, [C.POINTER(cvtx_P3D), bsv_V3f, _VF, _f]),
    "cvtx_P3D_S2S_dvort": (bsv_V3f, [C.POINTER(cvtx_P3D), C.POINTER(cvtx_P3D), _VF, _f]),
    "cvtx_P3D_S2S_visc_dvort": (bsv_V3f, [C.POINTER(cvtx_P3D), C.POINTER(cvtx_P3D), _VF, _f, _f]),
    "cvtx_P3D_S2S_vort": (bsv_V3f, [C.POINTER(cvtx_P3D), bsv_V3f, _VF, _f]),
    "cvtx_P3D_S2M_vel": (None, [_vp, _vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_S2M_dvort": (None, [_vp, _vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_S2M_visc_dvort": (None, [_vp, _vp, _i, _vp, _VF, _f, _f]),
    "cvtx_P3D_S2M_vort": (None, [_vp, _vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_M2S_vel": (bsv_V3f, [_vp, _i, bsv_V3f, _VF, _f]),
    "cvtx_P3D_M2S_dvort": (bsv_V3f, [_vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_M2S_visc_dvort": (bsv_V3f, [_vp, _i, _vp, _VF, _f, _f]),
    "cvtx_P3D_M2S_vort": (bsv_V3f, [_vp, _i, bsv_V3f, _VF, _f]),
    "cvtx_P3D_M2M_vel": (None, [_vp, _i, _vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_M2M_dvort": (None, [_vp, _i, _vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_M2M_visc_dvort": (None, [_vp, _i, _vp, _i, _vp, _VF, _f, _f]),
    "cvtx_P3D_M2M_vort": (None, [_vp, _i, _vp, _i, _vp, _VF, _f]),
    "cvtx_P3D_redistribute_on_grid": (_i, [_vp, _i, _vp, _i, _vp, _f, _f]),
    "cvtx_P3D_pedrizzetti_relaxation": (None, [_vp, _i, _f, _VF, _f]),
    "cvtx_F3D_S2S_vel": (bsv_V3f, [C.POINTER(cvtx_F3D), bsv_V3f]),
    "cvtx_F3D_S2S_dvort": (bsv_V3f, [C.POINTER(cvtx_F3D), C.POINTER(cvtx_P3D)]),
    "cvtx_F3D_M2S_vel": (bsv_V3f, [_vp, _i, bsv_V3f]),
    "cvtx_F3D_M2S_dvort": (bsv_V3f, [_vp, _i, _vp]),
    "cvtx_F3D_M2M_vel": (None, [_vp, _i, _vp, _i, _vp]),
    "cvtx_F3D_M2M_dvort": (None, [_vp, _i, _vp, _i, _vp]),
    "cvtx_F3D_inf_mtrx": (None, [_vp, _i, _vp, _vp, _i, _vp]),
    "cvtx_P2D_S2S_vel": (bsv_V2f, [C.POINTER(cvtx_P2D), bsv_V2f, _VF, _f]),
    "cvtx_P2D_S2M_vel": (None, [_vp, _vp, _i, _vp, _VF, _f]),
    "cvtx_P2D_M2S_vel": (bsv_V2f, [_vp, _i, bsv_V2f, _VF, _f]),
    "cvtx_P2D_M2M_vel": (None, [_vp, _i, _vp, _i, _vp, _VF, _f]),
    "cvtx_P2D_S2S_visc_dvort": (_f, [C.POINTER(cvtx_P2D), C.POINTER(cvtx_P2D), _VF, _f, _f]),
    "cvtx_P2D_S2M_visc_dvort": (None, [_vp, _vp, _i, _vp, _VF, _f, _f]),
    "cvtx_P2D_M2S_visc_dvort": (_f, [_vp, _i, _vp, _VF, _f, _f]),
    "cvtx_P2D_M2M_visc_dvort": (None, [_vp, _i, _vp, _i, _vp, _VF, _f, _f]),
    "cvtx_P2D_redistribute_on_grid": (_i, [_vp, _i, _vp, _i, _vp, _f, _f]),
}

class cvtx_gb300_p3d_problem(C.Structure):
    _fields_ = [("src", C.c_void_p), ("n_src", C.c_int), ("tgt", C.c_void_p),
                ("tgt_stride", C.c_int), ("n_tgt", C.c_int), ("vel_out", C.c_void_p),
                ("dvort_out", C.c_void_p), ("sigma", C.c_float)]


class cvtx_gb300_request(C.Structure):
    _fields_ = [("kind", C.c_int), ("reg", C.c_int), ("sigma", C.c_float), ("dt", C.c_float),
                ("n_steps", C.c_int), ("n", C.c_int), ("n_tgt", C.c_int),
                ("state_in", C.c_void_p), ("tgt_in", C.c_void_p),
                ("state_out", C.c_void_p), ("vel_out", C.c_void_p)]


class cvtx_gb300_server_stats(C.Structure):
    _fields_ = [(k, C.c_ulonglong) for k in
                ("submitted", "completed", "rejected", "failed", "queued", "in_flight")] + \
               [(k, C.c_double) for k in
                ("p50_ms", "p99_ms", "mean_ms", "max_ms", "queue_p50_ms", "queue_p99_ms",
                 "interactions", "span_s")] + \
               [(k, C.c_ulonglong) for k in
                ("hbm_budget", "hbm_used", "hbm_peak", "kernel_launches")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# GB300 extensions (include/cvortex/cvtx_gb300.h).
_EXT_SIGS = {
    "cvtx_gb300_last_error": (C.c_char_p, []),
    "cvtx_gb300_clear_error": (None, []),
    "cvtx_gb300_kernel_launches": (C.c_ulonglong, []),
    "cvtx_gb300_gaussian_rho_c": (_f, []),
    "cvtx_gb300_set_gaussian_rho_c": (None, [_f]),
    "cvtx_gb300_P3D_M2M_vel_dvort": (_i, [_vp, _i, _vp, _vp, _VF, _f]),
    "cvtx_gb300_dev_P3D_M2M": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp, _i, _f, _vp]),
    "cvtx_gb300_dev_P3D_M2M_visc": (_i, [_vp, _i, _vp, _i, _i, _vp, _i, _f, _f, _vp]),
    "cvtx_gb300_dev_P3D_M2M_ws_bytes": (C.c_longlong, [_i, _i, _i, _i, _i, _i]),
    "cvtx_gb300_dev_P3D_M2M_vort": (_i, [_vp, _i, _vp, _i, _i, _vp, _i, _f, _vp]),
    "cvtx_gb300_dev_P2D_M2M_vel": (_i, [_vp, _i, _vp, _i, _vp, _i, _f, _vp]),
    "cvtx_gb300_dev_P2D_M2M_visc": (_i, [_vp, _i, _vp, _i, _vp, _i, _f, _f, _vp]),
    "cvtx_gb300_dev_F3D_inf_mtrx": (_i, [_vp, _i, _vp, _vp, _i, _vp, _vp]),
    "cvtx_gb300_dev_F3D_M2M_vel": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp]),
    "cvtx_gb300_dev_F3D_M2M_dvort": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp]),
    "cvtx_gb300_dev_P3D_M2M_noalloc": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp, _i, _f, _vp]),
    "cvtx_gb300_p3d_num_configs": (_i, []),
    "cvtx_gb300_p3d_config_info": (_i, [_i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "cvtx_gb300_size_bucket": (_i, [_i]),
    "cvtx_gb300_p3d_set_tuned": (_i, [_i, _i, _i, _i]),
    "cvtx_gb300_p3d_current_config": (_i, [_i, _i, _i]),
    "cvtx_gb300_batch_create": (_vp, [C.POINTER(cvtx_gb300_p3d_problem), _i, _i, _i]),
    "cvtx_gb300_batch_tune": (_i, [_vp, _i]),
    "cvtx_gb300_batch_capture": (_i, [_vp]),
    "cvtx_gb300_batch_run": (_i, [_vp, _vp]),
    "cvtx_gb300_batch_status": (_i, [_vp]),
    "cvtx_gb300_batch_info": (_i, [_vp, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i),
                                   C.POINTER(_i), C.POINTER(_i), C.POINTER(C.c_double)]),
    "cvtx_gb300_batch_destroy": (None, [_vp]),
    "cvtx_gb300_dev_P3D_step": (_i, [_vp, _i, _vp, _vp, _i, _f, _f, _vp]),
    "cvtx_gb300_server_create": (_vp, [_i, C.c_ulonglong, _i]),
    "cvtx_gb300_server_submit": (C.c_ulonglong, [_vp, C.POINTER(cvtx_gb300_request)]),
    "cvtx_gb300_server_replay": (_i, [_vp, C.POINTER(cvtx_gb300_request),
                                      C.POINTER(C.c_double), _i, C.POINTER(C.c_ulonglong)]),
    "cvtx_gb300_server_wait": (_i, [_vp, C.c_ulonglong, C.c_double]),
    "cvtx_gb300_server_drain": (_i, [_vp, C.c_double]),
    "cvtx_gb300_server_request_info": (_i, [_vp, C.c_ulonglong, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]),
    "cvtx_gb300_server_stats_get": (_i, [_vp, C.POINTER(cvtx_gb300_server_stats)]),
    "cvtx_gb300_server_reset_stats": (None, [_vp]),
    "cvtx_gb300_server_inject_alloc_failures": (None, [_vp, _i]),
    "cvtx_gb300_server_destroy": (None, [_vp]),
    "cvtx_gb300_selftest_withheld_wait": (_i, [C.c_double]),
    "cvtx_gb300_dev_status": (_i, [_vp]),
    "cvtx_gb300_probe_fp32_tflops": (_i, [_i, C.POINTER(C.c_double)]),
    "cvtx_gb300_probe_fp32_detail": (_i, [_i, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "cvtx_gb300_probe_fp32_mix": (_i, [_i, _i, _i, C.POINTER(C.c_double)]),
    "cvtx_gb300_dev_pack_P3D": (_i, [_vp, _i, _vp, _vp]),
    "cvtx_gb300_dev_pack_V3f": (_i, [_vp, _i, _vp, _vp]),
}

REFERENCE_SYMBOLS = tuple(_SIGS)
EXTENSION_SYMBOLS = tuple(_EXT_SIGS)


def bind(lib: C.CDLL, sigs: dict) -> None:
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def load_library(path: Path | str | None = None, extensions: bool = True) -> C.CDLL:
    """Load and bind the library; ``extensions=False`` binds only the
    reference ABI (for loading the reference build itself)."""
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -m cvortex_gb300.build` "
            "(or __graft_entry__.build()); there is no fallback implementation")
    lib = C.CDLL(str(p))
    bind(lib, _SIGS)
    if extensions:
        bind(lib, _EXT_SIGS)
    return lib


# ---- numpy helpers ----------------------------------------------------------
def ptr_array(arr: np.ndarray) -> np.ndarray:
    """Array of record pointers into a contiguous structured array."""
    assert arr.flags["C_CONTIGUOUS"]
    n = arr.shape[0]
    return (np.uint64(arr.ctypes.data) + np.arange(n, dtype=np.uint64) * np.uint64(arr.itemsize))


def _addr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


def make_p3d(coord, vort, vol) -> np.ndarray:
    coord = np.asarray(coord, np.float32)
    out = np.zeros(coord.shape[0], P3D_DTYPE)
    out["coord"] = coord
    out["vorticity"] = np.asarray(vort, np.float32)
    out["volume"] = np.asarray(vol, np.float32)
    return out


def make_p2d(coord, vort, area) -> np.ndarray:
    coord = np.asarray(coord, np.float32)
    out = np.zeros(coord.shape[0], P2D_DTYPE)
    out["coord"] = coord
    out["vorticity"] = np.asarray(vort, np.float32)
    out["area"] = np.asarray(area, np.float32)
    return out


def make_f3d(start, end, strength) -> np.ndarray:
    start = np.asarray(start, np.float32)
    out = np.zeros(start.shape[0], F3D_DTYPE)
    out["start"] = start
    out["end"] = np.asarray(end, np.float32)
    out["strength"] = np.asarray(strength, np.float32)
    return out


class Cvtx:
    """numpy front end over the C ABI (one instance per loaded library)."""

    def __init__(self, path: Path | str | None = None, extensions: bool = True):
        self.lib = load_library(path, extensions)
        self._vf = {}

    # -- lifecycle / accelerators
    def initialise(self):
        self.lib.cvtx_initialise()

    def finalise(self):
        self.lib.cvtx_finalise()

    def num_accelerators(self) -> int:
        return self.lib.cvtx_num_accelerators()

    def set_accelerated(self, on: bool):
        for i in range(self.lib.cvtx_num_accelerators()):
            (self.lib.cvtx_accelerator_enable if on else self.lib.cvtx_accelerator_disable)(i)

    def launches(self) -> int:
        return int(self.lib.cvtx_gb300_kernel_launches())

    def last_error(self) -> str:
        return (self.lib.cvtx_gb300_last_error() or b"").decode()

    def vortfunc(self, name: str) -> cvtx_VortFunc:
        if name not in self._vf:
            self._vf[name] = getattr(self.lib, f"cvtx_VortFunc_{name}")()
        return self._vf[name]

    # -- M2M conveniences (sources as structured arrays, results as float32)
    def p3d_vel(self, src, mes, reg, sigma):
        p = ptr_array(src)
        mes = np.ascontiguousarray(mes, np.float32)
        out = np.zeros((mes.shape[0], 3), np.float32)
        self.lib.cvtx_P3D_M2M_vel(_addr(p), len(src), _addr(mes), mes.shape[0], _addr(out),
                                  C.byref(self.vortfunc(reg)), sigma)
        return out

    def p3d_dvort(self, src, ind, reg, sigma, same=False):
        p = ptr_array(src)
        q = p if same else ptr_array(ind)
        n_ind = len(src) if same else len(ind)
        out = np.zeros((n_ind, 3), np.float32)
        self.lib.cvtx_P3D_M2M_dvort(_addr(p), len(src), _addr(q), n_ind, _addr(out),
                                    C.byref(self.vortfunc(reg)), sigma)
        return out

    def p3d_visc(self, src, ind, reg, sigma, nu, same=False):
        p = ptr_array(src)
        q = p if same else ptr_array(ind)
        n_ind = len(src) if same else len(ind)
        out = np.zeros((n_ind, 3), np.float32)
        self.lib.cvtx_P3D_M2M_visc_dvort(_addr(p), len(src), _addr(q), n_ind, _addr(out),
                                         C.byref(self.vortfunc(reg)), sigma, nu)
        return out

    def p3d_vort(self, src, mes, reg, sigma):
        p = ptr_array(src)
        mes = np.ascontiguousarray(mes, np.float32)
        out = np.zeros((mes.shape[0], 3), np.float32)
        self.lib.cvtx_P3D_M2M_vort(_addr(p), len(src), _addr(mes), mes.shape[0], _addr(out),
                                   C.byref(self.vortfunc(reg)), sigma)
        return out

    def p3d_vel_dvort(self, src, reg, sigma):
        p = ptr_array(src)
        vel = np.zeros((len(src), 3), np.float32)
        dv = np.zeros((len(src), 3), np.float32)
        rc = self.lib.cvtx_gb300_P3D_M2M_vel_dvort(_addr(p), len(src), _addr(vel), _addr(dv),
                                                   C.byref(self.vortfunc(reg)), sigma)
        if rc != 0:
            raise RuntimeError(f"cvtx_gb300_P3D_M2M_vel_dvort failed ({rc}): {self.last_error()}")
        return vel, dv

    def p2d_vel(self, src, mes, reg, sigma):
        p = ptr_array(src)
        mes = np.ascontiguousarray(mes, np.float32)
        out = np.zeros((mes.shape[0], 2), np.float32)
        self.lib.cvtx_P2D_M2M_vel(_addr(p), len(src), _addr(mes), mes.shape[0], _addr(out),
                                  C.byref(self.vortfunc(reg)), sigma)
        return out

    def p2d_visc(self, src, ind, reg, sigma, nu, same=False):
        p = ptr_array(src)
        q = p if same else ptr_array(ind)
        n_ind = len(src) if same else len(ind)
        out = np.zeros(n_ind, np.float32)
        self.lib.cvtx_P2D_M2M_visc_dvort(_addr(p), len(src), _addr(q), n_ind, _addr(out),
                                         C.byref(self.vortfunc(reg)), sigma, nu)
        return out

    def f3d_vel(self, fil, mes):
        p = ptr_array(fil)
        mes = np.ascontiguousarray(mes, np.float32)
        out = np.zeros((mes.shape[0], 3), np.float32)
        self.lib.cvtx_F3D_M2M_vel(_addr(p), len(fil), _addr(mes), mes.shape[0], _addr(out))
        return out

    def f3d_dvort(self, fil, ind):
        p = ptr_array(fil)
        q = ptr_array(ind)
        out = np.zeros((len(ind), 3), np.float32)
        self.lib.cvtx_F3D_M2M_dvort(_addr(p), len(fil), _addr(q), len(ind), _addr(out))
        return out

    def f3d_inf_mtrx(self, fil, mes, dirs):
        p = ptr_array(fil)
        mes = np.ascontiguousarray(mes, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        out = np.zeros((mes.shape[0], len(fil)), np.float32)
        self.lib.cvtx_F3D_inf_mtrx(_addr(p), len(fil), _addr(mes), _addr(dirs), mes.shape[0],
                                   _addr(out))
        return out

    def relax(self, particles, fdt, reg, sigma):
        p = ptr_array(particles)
        self.lib.cvtx_P3D_pedrizzetti_relaxation(_addr(p), len(particles), fdt,
                                                 C.byref(self.vortfunc(reg)), sigma)
