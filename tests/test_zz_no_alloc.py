"""The allocation-free entry point cvtx_gb300_dev_P3D_M2M_noalloc.

It serves callers that cannot let the library allocate device memory: a
solver whose GPU memory all comes from one pool reserved at start-up, or a
time-stepping loop that cannot take the latency and synchronisation of
cudaMalloc / cudaFree. Its split partial sums live in a fixed 32 MiB scratch
area inside the library image instead of a workspace allocated on demand.

Checked here, through the C ABI on device buffers: on two calls in a row it
matches the existing entry point cvtx_gb300_dev_P3D_M2M within the parity
tolerance (including a case where the scratch caps the number of source
splits); its second call changes the device's free memory by nothing; and
target counts beyond its limit are rejected without a launch. This file is
collected last, and it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from cvortex_gb300 import workloads
from oracle import exact
from parity import TOL

pytestmark = pytest.mark.gpu
REG = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}
MAX_TARGETS = 233_016


def _records(p):
    rec = np.zeros((len(p), 8), np.float32)
    rec[:, 0:3] = p["coord"]
    rec[:, 3] = p["volume"]
    rec[:, 4:7] = p["vorticity"]
    return rec


@pytest.mark.parametrize("reg, ops, n_src, n_tgt", [
    ("winckelmans", "fused", 40_000, 3_000),
    ("gaussian", "dvort", 20_000, 9_000),
    ("singular", "vel", 5_000, 20_000),
    ("winckelmans", "fused", 60_000, 200_000),   # scratch caps the split count
    ("gaussian", "fused", 300_000, 40),           # the few-target form
])
def test_noalloc_matches_existing_entry_point(gpu, reg, ops, n_src, n_tgt):
    import torch
    lib = gpu.lib
    src = torch.from_numpy(_records(workloads.vortex_ring(n_src, seed=61))).cuda()
    tgt = torch.from_numpy(_records(workloads.vortex_ring(n_tgt, seed=62))).cuda()
    want_vel = ops in ("fused", "vel")
    want_dv = ops in ("fused", "dvort")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def buf():
        return torch.full((n_tgt, 3), 7.0, dtype=torch.float32, device="cuda")

    def ptr(t):
        return t.data_ptr() if t is not None else None

    ev, ed = (buf() if want_vel else None), (buf() if want_dv else None)
    rc = lib.cvtx_gb300_dev_P3D_M2M(src.data_ptr(), n_src, tgt.data_ptr(), 2, n_tgt, ptr(ev),
                                    ptr(ed), REG[reg], 0.05, stream)
    assert rc == 0, gpu.last_error()
    torch.cuda.synchronize()
    nv, nd = (buf() if want_vel else None), (buf() if want_dv else None)
    for call in range(2):
        for t in (nv, nd):
            if t is not None:
                t.fill_(7.0)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.cvtx_gb300_dev_P3D_M2M_noalloc(src.data_ptr(), n_src, tgt.data_ptr(), 2, n_tgt,
                                                ptr(nv), ptr(nd), REG[reg], 0.05, stream)
        assert rc == 0, gpu.last_error()
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        for got, want in ((nv, ev), (nd, ed)):
            if got is None:
                continue
            g, w = got.cpu().numpy(), want.cpu().numpy()
            assert np.all(np.isfinite(g))
            assert exact.rel_l2(g, w) <= TOL, (call, exact.rel_l2(g, w))


def test_noalloc_rejects_too_many_targets(gpu):
    import torch
    lib = gpu.lib
    small = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    out = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    before = gpu.launches()
    rc = lib.cvtx_gb300_dev_P3D_M2M_noalloc(small.data_ptr(), 4, small.data_ptr(), 2,
                                            MAX_TARGETS + 1, out.data_ptr(), None, 1, 0.05,
                                            None)
    assert rc == -1
    assert gpu.launches() == before
    assert str(MAX_TARGETS) in gpu.last_error()
    lib.cvtx_gb300_clear_error()
