"""Parity at the full sizes of the benchmark configurations.

* The headline: P3D velocity + stretching, Winckelmans, sigma 0.05, uniform
  cube of N = 1,000,000 (reference src/P3D.cpp:343-366, 387-410). Every
  target is computed on the GPU; 2,048 sampled targets are checked against
  the oracle (the reference CPU formulation) over all 10^6 sources, 256 of
  them against FP64 as well; linearity in vorticity is checked on every
  target.
* The benchmark's 512-problem batch (sizes log-uniform on [1,000, 50,000],
  the same seeds): every problem against the per-call device API, and 16
  problems (the three largest among them) on sampled targets against the
  oracle.
* One served P3D request of 200,000 particles: its velocity and stretching
  (one step) on sampled targets against the oracle.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from cvortex_gb300 import abi, serve, workloads
from oracle import exact
from parity import TOL, same_up_to_rounding

pytestmark = pytest.mark.gpu

SIG = 0.05


def _records(p):
    r = np.zeros((len(p), 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7] = p["coord"], p["volume"], p["vorticity"]
    return r


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_headline_cube_1m_winckelmans(gpu):
    import torch
    n = 1_000_000
    p = workloads.uniform_cube(n)
    rec = torch.from_numpy(_records(p)).cuda()
    vel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    sh = _stream(torch)
    assert gpu.lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n, vel.data_ptr(),
                                          dv.data_ptr(), 1, SIG, sh) == 0
    assert gpu.lib.cvtx_gb300_dev_status(sh) == 0
    v, d = vel.cpu().numpy(), dv.cpu().numpy()
    assert np.all(np.isfinite(v)) and np.all(np.isfinite(d))
    idx = np.sort(np.random.Generator(np.random.PCG64(41)).choice(n, 2048, replace=False))
    sub = p[idx].copy()
    rv = oracle.p3d_vel(p, sub["coord"], "winckelmans", SIG)
    rd = oracle.p3d_dvort(p, sub, "winckelmans", SIG)
    assert exact.rel_l2(v[idx], rv) <= TOL
    assert exact.rel_l2(d[idx], rd) <= TOL
    f = idx[::8]
    fs = p[f].copy()
    ev, ed = oracle.exact_p3d_vel_dvort(p, fs["coord"], fs["vorticity"], "winckelmans", SIG)
    assert exact.rel_l2(v[f], ev) <= TOL and exact.rel_l2(d[f], ed) <= TOL
    # vel is linear and dvort quadratic in vorticity: x2 is exact in FP32
    rec[:, 4:7] *= 2
    assert gpu.lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n, vel.data_ptr(),
                                          dv.data_ptr(), 1, SIG, sh) == 0
    np.testing.assert_array_equal(vel.cpu().numpy(), 2 * v)
    np.testing.assert_array_equal(dv.cpu().numpy(), 4 * d)


def test_batch_512_benchmark_problems(gpu):
    import torch
    lib = gpu.lib
    sizes = workloads.batch_sizes(512)
    keep, probs = [], []
    for i, n in enumerate(sizes):
        n = int(n)
        p = workloads.uniform_cube(n, seed=10_000 + i)
        rec = torch.from_numpy(_records(p)).cuda()
        v = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
        d = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
        keep.append((p, rec, v, d))
        probs.append(abi.cvtx_gb300_p3d_problem(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                v.data_ptr(), d.data_ptr(), SIG))
    arr = (abi.cvtx_gb300_p3d_problem * len(probs))(*probs)
    b = lib.cvtx_gb300_batch_create(arr, len(probs), 1, 3)
    assert b, gpu.last_error()
    sh = _stream(torch)
    try:
        assert lib.cvtx_gb300_batch_tune(b, 1) == 0
        assert lib.cvtx_gb300_batch_capture(b) == 0
        assert lib.cvtx_gb300_batch_run(b, sh) == 0
        torch.cuda.synchronize()
        assert lib.cvtx_gb300_batch_status(b) == 0
    finally:
        lib.cvtx_gb300_batch_destroy(b)
    ev = torch.empty((int(sizes.max()), 3), dtype=torch.float32, device="cuda")
    ed = torch.empty_like(ev)
    for p, rec, v, d in keep:
        n = len(p)
        assert lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n, ev.data_ptr(),
                                          ed.data_ptr(), 1, SIG, sh) == 0
        torch.cuda.synchronize()
        # the batch's self-interaction part and the per-call kernels differ
        # in summation order only
        same_up_to_rounding(p, "winckelmans", "vel", v.cpu().numpy(), ev[:n].cpu().numpy(), n, SIG)
        same_up_to_rounding(p, "winckelmans", "dvort", d.cpu().numpy(), ed[:n].cpu().numpy(), n,
                            SIG)
        assert exact.rel_l2(v.cpu().numpy(), ev[:n].cpu().numpy()) <= 1e-6
        assert exact.rel_l2(d.cpu().numpy(), ed[:n].cpu().numpy()) <= 1e-6
    order = np.argsort(sizes)
    rng = np.random.Generator(np.random.PCG64(42))
    chk = list(order[-3:]) + list(rng.choice(order[:-3], 13, replace=False))
    for i in chk:
        p, _, v, d = keep[i]
        ti = np.sort(rng.choice(len(p), min(len(p), 512), replace=False))
        sub = p[ti].copy()
        assert exact.rel_l2(v.cpu().numpy()[ti], oracle.p3d_vel(p, sub["coord"], "winckelmans",
                                                                SIG)) <= TOL, i
        assert exact.rel_l2(d.cpu().numpy()[ti], oracle.p3d_dvort(p, sub, "winckelmans", SIG)) <= TOL, i


def test_served_p3d_200k(gpu):
    """One step of a served 200,000-particle request: the step's velocity
    and the updated vorticity (alpha + dt * dvort) against the oracle."""
    n, dt = 200_000, 1e-3
    p = workloads.uniform_cube(n, seed=51)
    with serve.Server(gpu.lib, n_slots=4) as srv:
        req = serve.Request.p3d(p, n_steps=1, dt=dt, reg=1, sigma=SIG)
        rid = srv.submit(req)
        assert rid
        assert srv.wait(rid, 120_000) == 0
    ti = np.sort(np.random.Generator(np.random.PCG64(43)).choice(n, 1024, replace=False))
    sub = p[ti].copy()
    rv = oracle.p3d_vel(p, sub["coord"], "winckelmans", SIG)
    rd = oracle.p3d_dvort(p, sub, "winckelmans", SIG)
    assert exact.rel_l2(req.vel_out[ti], rv) <= TOL
    # the update's FP32 rounding of alpha (~6e-8) is far below dt * |dvort|
    a1 = sub["vorticity"].astype(np.float64) + dt * rd.astype(np.float64)
    assert exact.rel_l2(req.state_out[ti, 4:7], a1) <= 1e-6
    x1 = sub["coord"].astype(np.float64) + dt * rv.astype(np.float64)
    assert exact.rel_l2(req.state_out[ti, 0:3], x1) <= 1e-6


@pytest.mark.parametrize("reg", ["singular", "winckelmans", "planetary", "gaussian"])
def test_every_configuration_on_every_target_ring_100k(gpu, reg):
    """The 100,000-particle ring through every launch configuration of the
    per-call P3D kernels (scalar and packed, every targets-per-thread and
    CTA shape, forced through the tuning table), each op, compared with the
    one-target-per-thread scalar kernel on every target: a fault confined to
    one packed lane or one target slot of a thread shows on 1/2 .. 1/6 of
    the targets. The scalar kernel itself is checked against the oracle on
    sampled targets."""
    import torch
    n = 100_000
    p = workloads.vortex_ring(n, seed=81)
    rec = torch.from_numpy(_records(p)).cuda()
    sh = _stream(torch)
    r = abi.REG_IDS[reg]
    bucket = gpu.lib.cvtx_gb300_size_bucket(n)
    n_cfg = gpu.lib.cvtx_gb300_p3d_num_configs()
    few_cfg = n_cfg - 1                  # the few-target form: not for 10^5 targets
    idx = np.sort(np.random.Generator(np.random.PCG64(82)).choice(n, 512, replace=False))
    sub = p[idx].copy()
    ref_v = oracle.p3d_vel(p, sub["coord"], reg, SIG)
    ref_d = oracle.p3d_dvort(p, sub, reg, SIG)

    def run(ops, cfg):
        v = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
        d = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
        assert gpu.lib.cvtx_gb300_p3d_set_tuned(r, ops, bucket, cfg) == 0
        try:
            assert gpu.lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                  v.data_ptr() if ops & 1 else None,
                                                  d.data_ptr() if ops & 2 else None,
                                                  r, SIG, sh) == 0
            assert gpu.lib.cvtx_gb300_dev_status(sh) == 0
        finally:
            gpu.lib.cvtx_gb300_p3d_set_tuned(r, ops, bucket, -1)
        return (v.cpu().numpy() if ops & 1 else None), (d.cpu().numpy() if ops & 2 else None)

    for ops in (1, 2, 3):
        base_v, base_d = run(ops, 0)
        if ops & 1:
            assert exact.rel_l2(base_v[idx], ref_v) <= TOL
        if ops & 2:
            assert exact.rel_l2(base_d[idx], ref_d) <= TOL
        for cfg in range(1, n_cfg):
            if cfg == few_cfg:
                continue
            v, d = run(ops, cfg)
            for name, got, base in (("vel", v, base_v), ("dvort", d, base_d)):
                if got is not None:
                    same_up_to_rounding(p, reg, name, got, base, (ops, cfg), SIG)
