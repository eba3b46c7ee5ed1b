"""Batched form (many independent P3D problems in one persistent launch,
problems from 4,096 particles in the self-interaction form): each
problem's result matches the per-call device API, the captured CUDA graph
replays deterministically, and tuning keeps results within tolerance."""
import ctypes as C

import numpy as np
import pytest

import oracle
from cvortex_gb300 import abi, workloads
from oracle import exact
from parity import TOL, same_up_to_rounding

pytestmark = pytest.mark.gpu


def _records(p):
    rec = np.zeros((len(p), 8), np.float32)
    rec[:, 0:3] = p["coord"]
    rec[:, 3] = p["volume"]
    rec[:, 4:7] = p["vorticity"]
    return rec


def _make(torch, sizes, ops, seed0=100):
    probs, keep = [], []
    for i, n in enumerate(sizes):
        p = workloads.uniform_cube(int(n), seed=seed0 + i)
        rec = torch.from_numpy(_records(p)).cuda()
        vel = torch.zeros((n, 3), dtype=torch.float32, device="cuda") if ops & 1 else None
        dv = torch.zeros((n, 3), dtype=torch.float32, device="cuda") if ops & 2 else None
        keep.append((p, rec, vel, dv))
        probs.append(abi.cvtx_gb300_p3d_problem(
            rec.data_ptr(), int(n), rec.data_ptr(), 2, int(n),
            vel.data_ptr() if vel is not None else None,
            dv.data_ptr() if dv is not None else None, 0.05))
    arr = (abi.cvtx_gb300_p3d_problem * len(probs))(*probs)
    return arr, keep


@pytest.mark.parametrize("reg, ops", [("winckelmans", 3), ("gaussian", 3), ("singular", 2),
                                      ("planetary", 1)])
def test_batch_matches_per_call(gpu, reg, ops):
    import torch
    lib = gpu.lib
    sizes = [1, 300, 1000, 2500, 257, 7000, 513, 30000, 4096, 12000]
    arr, keep = _make(torch, sizes, ops)
    b = lib.cvtx_gb300_batch_create(arr, len(sizes), abi.REG_IDS[reg], ops)
    assert b, gpu.last_error()
    try:
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        assert lib.cvtx_gb300_batch_run(b, stream) == 0
        torch.cuda.synchronize()
        assert lib.cvtx_gb300_batch_status(b) == 0
        for p, rec, vel, dv in keep:
            n = len(p)
            ev = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
            ed = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
            rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                            ev.data_ptr() if ops & 1 else None,
                                            ed.data_ptr() if ops & 2 else None,
                                            abi.REG_IDS[reg], 0.05, stream)
            assert rc == 0
            torch.cuda.synchronize()
            # problems from 4,096 particles run in the self-interaction
            # form in the batch: the two differ in summation order only
            if ops & 1:
                same_up_to_rounding(p, reg, "vel", vel.cpu().numpy(), ev.cpu().numpy(), n, 0.05)
            if ops & 2:
                same_up_to_rounding(p, reg, "dvort", dv.cpu().numpy(), ed.cpu().numpy(), n, 0.05)
        # one problem against the oracle directly
        p, rec, vel, dv = keep[6]
        if ops & 1:
            assert exact.rel_l2(vel.cpu().numpy(), oracle.p3d_vel(p, p["coord"], reg, 0.05)) <= TOL
    finally:
        lib.cvtx_gb300_batch_destroy(b)


def test_batch_graph_replay_and_tuning(gpu):
    import torch
    lib = gpu.lib
    rng = np.random.Generator(np.random.PCG64(9))
    sizes = np.exp(rng.uniform(np.log(500), np.log(20000), 24)).astype(int)
    arr, keep = _make(torch, sizes, 3, seed0=300)
    b = lib.cvtx_gb300_batch_create(arr, len(sizes), 1, 3)
    assert b, gpu.last_error()
    try:
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        assert lib.cvtx_gb300_batch_run(b, stream) == 0
        torch.cuda.synchronize()
        first = [(v.cpu().numpy().copy(), d.cpu().numpy().copy()) for _, _, v, d in keep]
        assert lib.cvtx_gb300_batch_capture(b) == 0
        g = C.c_int()
        lib.cvtx_gb300_batch_info(b, None, None, None, None, C.byref(g), None)
        assert g.value == 1
        for _ in range(2):
            for _, _, v, d in keep:
                v.fill_(7.0)
                d.fill_(7.0)
            assert lib.cvtx_gb300_batch_run(b, stream) == 0
            torch.cuda.synchronize()
            for (v0, d0), (_, _, v, d) in zip(first, keep):
                np.testing.assert_array_equal(v.cpu().numpy(), v0)
                np.testing.assert_array_equal(d.cpu().numpy(), d0)
        assert lib.cvtx_gb300_batch_tune(b, 1) == 0
        assert lib.cvtx_gb300_batch_capture(b) == 0
        assert lib.cvtx_gb300_batch_run(b, stream) == 0
        torch.cuda.synchronize()
        assert lib.cvtx_gb300_batch_status(b) == 0
        for (v0, d0), (_, _, v, d) in zip(first, keep):
            assert exact.rel_l2(v.cpu().numpy(), v0) <= 1e-6
            assert exact.rel_l2(d.cpu().numpy(), d0) <= 1e-6
    finally:
        lib.cvtx_gb300_batch_destroy(b)


BATCH_CHILD = r"""
import sys
import numpy as np, torch
sys.path.insert(0, sys.argv[2])
sys.path.insert(0, sys.argv[3])
from cvortex_gb300 import abi
from test_gpu_batch import _make
cv = abi.Cvtx(); cv.initialise()
lib = cv.lib
sizes = [5000, 12000, 30000, 700]
arr, keep = _make(torch, sizes, 3, seed0=500)
b = lib.cvtx_gb300_batch_create(arr, len(sizes), 1, 3)
assert b, cv.last_error()
sh = torch.cuda.current_stream().cuda_stream
import ctypes as C
assert lib.cvtx_gb300_batch_run(b, C.c_void_p(sh)) == 0
torch.cuda.synchronize()
assert lib.cvtx_gb300_batch_status(b) == 0, cv.last_error()
lib.cvtx_gb300_batch_destroy(b)
np.savez(sys.argv[1], *[np.concatenate([v.cpu().numpy(), d.cpu().numpy()], 1) for _, _, v, d in keep])
"""


def _batch_child(tmp_path, tag, env):
    import os
    import subprocess
    import sys
    from pathlib import Path
    out = tmp_path / f"batch_{tag}.npz"
    root = Path(__file__).resolve().parents[1]
    res = subprocess.run([sys.executable, "-c", BATCH_CHILD, str(out), str(root),
                          str(root / "tests")], cwd=root, env=dict(os.environ, **env),
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    z = np.load(out)
    return [z[f"arr_{i}"] for i in range(len(z.files))]


def test_batch_self_part_fallbacks(gpu, tmp_path):
    """The batch's self-interaction part switched off (CVTX_GB300_SYM_MIN=0)
    and its tables not allocatable (CVTX_GB300_WS_LIMIT below them: an
    injected out-of-memory) both leave every problem to the ordered-pair
    items, bit for bit the same; with the part, the results agree within the
    FP32 bound."""
    with_part = _batch_child(tmp_path, "sym", {})
    ordered = _batch_child(tmp_path, "ordered", {"CVTX_GB300_SYM_MIN": "0"})
    limited = _batch_child(tmp_path, "limited", {"CVTX_GB300_WS_LIMIT": str(16 << 20)})
    for a, c in zip(ordered, limited):
        np.testing.assert_array_equal(a, c)
    assert any(not np.array_equal(a, c) for a, c in zip(with_part, ordered))
    for a, c in zip(with_part, ordered):
        assert exact.rel_l2(a, c) <= 1e-6
