"""Calling the library's redistribution entry points from numpy arrays."""
import ctypes as C

import numpy as np

from cvortex_gb300 import abi


def p3d(lib, particles, fname, gd, negligible, max_out, null_output=False):
    ptrs = abi.ptr_array(particles)
    out = np.zeros(max(max_out, 1), abi.P3D_DTYPE)
    rf = getattr(lib, f"cvtx_RedistFunc_{fname}")()
    n = lib.cvtx_P3D_redistribute_on_grid(ptrs.ctypes.data, len(particles),
                                          None if null_output else out.ctypes.data, max_out,
                                          C.byref(rf), gd, negligible)
    return n, out[:min(n, max_out)]


def p2d(lib, particles, fname, gd, negligible, max_out, null_output=False):
    ptrs = abi.ptr_array(particles)
    out = np.zeros(max(max_out, 1), abi.P2D_DTYPE)
    rf = getattr(lib, f"cvtx_RedistFunc_{fname}")()
    n = lib.cvtx_P2D_redistribute_on_grid(ptrs.ctypes.data, len(particles),
                                          None if null_output else out.ctypes.data, max_out,
                                          C.byref(rf), gd, negligible)
    return n, out[:min(n, max_out)]
