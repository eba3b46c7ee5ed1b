"""cvortex_gb300 -- GB300-native (sm_103a) all-pairs vortex interactions behind
cvortex's unchanged cvtx_ C ABI.

The product is ``lib/libcvortex.so`` (C ABI; headers in ``include/cvortex``).
This package builds it (``cvortex_gb300.build``) and mirrors its interface in
Python through ctypes (``cvortex_gb300.abi``).
"""
from .abi import (  # noqa: F401
    Cvtx, F3D_DTYPE, P2D_DTYPE, P3D_DTYPE, REG_IDS, LIB_PATH, load_library, make_f3d, make_p2d,
    make_p3d, ptr_array,
)
