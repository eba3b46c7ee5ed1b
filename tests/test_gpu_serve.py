"""Serving loop on the GPU: a served request's velocity and state after its
device-resident steps match the oracle (restated reference CPU path) within
the parity bar, multi-step state matches the same steps taken through the
plain C ABI, and every result is bit-identical alone and in a mix of
concurrent requests of all kinds."""
import numpy as np
import pytest

import oracle
from cvortex_gb300 import serve, workloads
from oracle import exact
from parity import TOL

pytestmark = pytest.mark.gpu

SIG = 0.05


@pytest.fixture()
def srv(gpu):
    with serve.Server(gpu.lib, n_slots=8, hbm_bytes=2 << 30) as s:
        yield s


def _run(srv, req, timeout_ms=120_000):
    rid = srv.submit(req)
    assert rid, "request refused"
    st = srv.wait(rid, timeout_ms)
    assert st == 0, f"request status {serve.STATUS.get(st, st)}"
    return req


@pytest.mark.parametrize("reg", ["winckelmans", "gaussian", "singular"])
def test_p3d_one_step_vs_oracle(srv, reg):
    p = workloads.uniform_cube(3000, seed=21)
    dt = np.float32(1e-3)
    req = _run(srv, serve.Request.p3d(p, n_steps=1, dt=float(dt), reg=serve.REG_IDS[reg],
                                      sigma=SIG))
    vel = oracle.p3d_vel(p, p["coord"], reg, SIG)
    dv = oracle.p3d_dvort(p, p, reg, SIG)
    if reg == "gaussian":
        # the reference's erf form cancels below rho_c: compare against FP64
        v64, d64 = oracle.exact_p3d_vel_dvort(p, p["coord"], p["vorticity"], reg, SIG)
        assert exact.rel_l2(req.vel_out, v64) <= TOL
        vel, dv = v64, d64
    else:
        assert exact.rel_l2(req.vel_out, vel) <= TOL
    # updated state against the FP64 update from the oracle's rates: the
    # bound is FP32 rounding of the state (~1e-7), while a wrong rate would
    # show at dt * |rate| / |state| ~ 1e-3
    x1 = p["coord"].astype(np.float64) + float(dt) * vel
    a1 = p["vorticity"].astype(np.float64) + float(dt) * dv
    assert exact.rel_l2(req.state_out[:, 0:3], x1) <= 1e-6
    assert exact.rel_l2(req.state_out[:, 4:7], a1) <= 1e-6
    assert np.array_equal(req.state_out[:, 3], p["volume"])


def test_p2d_one_step_vs_oracle(srv):
    p = workloads.gaussian_patch_2d(4000, seed=22)
    req = _run(srv, serve.Request.p2d(p, n_steps=1, dt=1e-3, reg=1, sigma=SIG))
    vel = oracle.p2d_vel(p, p["coord"], "winckelmans", SIG)
    assert exact.rel_l2(req.vel_out, vel) <= TOL
    x1 = p["coord"].astype(np.float64) + 1e-3 * vel
    assert exact.rel_l2(req.state_out[:, 0:2], x1) <= 1e-6
    assert np.array_equal(req.state_out[:, 2], p["vorticity"])


def test_f3d_one_step_vs_oracle(srv):
    f = workloads.wake_sheet(1500, seed=23)
    pts = workloads.sheet_targets(2500, seed=24)
    req = _run(srv, serve.Request.f3d(f, pts, n_steps=1, dt=1e-3))
    vel = oracle.f3d_vel(f, pts)
    assert exact.rel_l2(req.vel_out, vel) <= TOL
    x1 = pts.astype(np.float64) + 1e-3 * vel
    assert exact.rel_l2(req.state_out[:, 0:3], x1) <= 1e-6


def test_p3d_ten_steps_vs_plain_abi(srv, gpu):
    """Ten resident steps equal ten plain ABI round trips (vel, dvort, host
    Euler update). A vortex ring keeps the flow smooth, so rounding
    differences between the two paths are not amplified by the steps (a
    random cloud with close pairs stretches them by orders of magnitude)."""
    p = workloads.vortex_ring(5000, seed=25)
    dt = np.float32(1e-3)
    req = _run(srv, serve.Request.p3d(p, n_steps=10, dt=float(dt), reg=1, sigma=SIG))
    q = p.copy()
    for _ in range(10):
        u = gpu.p3d_vel(q, q["coord"], "winckelmans", SIG)
        w = gpu.p3d_dvort(q, q, "winckelmans", SIG, same=True)
        q["coord"] = q["coord"] + dt * u
        q["vorticity"] = q["vorticity"] + dt * w
    # the two paths round the FP32 state differently (fused multiply-add on
    # the device, split partition): agreement to the parity bar
    assert exact.rel_l2(req.state_out[:, 0:3], q["coord"]) <= 1e-6
    assert exact.rel_l2(req.state_out[:, 4:7], q["vorticity"]) <= TOL
    assert exact.rel_l2(req.vel_out, u) <= TOL


def _mix(seed, count=24):
    rng = np.random.Generator(np.random.PCG64(seed))
    reqs = []
    for i in range(count):
        kind = int(rng.choice(3, p=workloads.SERVE_MIX))
        n = int(np.exp(rng.uniform(np.log(300), np.log(40_000))))
        a, b = workloads.serve_request_arrays(kind, n, 1000 + i)
        if kind == 0:
            reqs.append(serve.Request.p3d(a, n_steps=3))
        elif kind == 1:
            reqs.append(serve.Request.p2d(a, n_steps=3))
        else:
            reqs.append(serve.Request.f3d(a, b, n_steps=3))
    return reqs


def _probe_requests():
    p3 = workloads.uniform_cube(20_000, seed=31)
    p2 = workloads.gaussian_patch_2d(30_000, seed=32)
    f, pts = workloads.wake_sheet(8000, seed=33), workloads.sheet_targets(12_000, seed=34)
    return [serve.Request.p3d(p3, n_steps=4), serve.Request.p2d(p2, n_steps=4),
            serve.Request.f3d(f, pts, n_steps=4), serve.Request.p3d(p3[:777], n_steps=4)]


def test_alone_equals_in_mix(srv):
    """Bitwise: each probe run alone on an idle server, then again submitted
    in the middle of a burst of concurrent requests of every kind."""
    alone = _probe_requests()
    for r in alone:
        _run(srv, r)
    mixed = _probe_requests()
    burst = _mix(7)
    ids = []
    for i, r in enumerate(burst):
        ids.append(srv.submit(r))
        if i % 6 == 3:
            ids.append(srv.submit(mixed[i // 6]))
    assert srv.drain(300_000)
    assert all(srv.wait(i, 0) == 0 for i in ids)
    s = srv.stats()
    assert s["failed"] == 0 and s["rejected"] == 0
    for a, m in zip(alone, mixed):
        assert np.array_equal(a.state_out, m.state_out)
        assert np.array_equal(a.vel_out, m.vel_out)


def test_budget_rejection_and_pinned_buffers(gpu):
    import torch
    with serve.Server(gpu.lib, n_slots=2, hbm_bytes=4 << 20) as s:
        big = serve.Request.p3d(workloads.uniform_cube(100_000, seed=41), n_steps=1)
        rid = s.submit(big)
        assert s.wait(rid, 60_000) == -1
        # pinned caller buffers are copied directly (no staging)
        p = workloads.uniform_cube(2000, seed=42)
        pageable = _run(s, serve.Request.p3d(p, n_steps=2))
        req = serve.Request.p3d(p, n_steps=2)
        pin_in = torch.from_numpy(req.state_in).pin_memory()
        pin_out = torch.empty_like(pin_in).pin_memory()
        pin_vel = torch.empty((len(p), 3), dtype=torch.float32).pin_memory()
        req.state_in, req.state_out, req.vel_out = pin_in.numpy(), pin_out.numpy(), pin_vel.numpy()
        _run(s, req)
        assert np.array_equal(req.state_out, pageable.state_out)
        assert np.array_equal(req.vel_out, pageable.vel_out)
        st = s.stats()
        assert st["rejected"] == 1 and st["completed"] == 2 and st["hbm_used"] == 0


def test_dev_p3d_step_matches_served_step(gpu, srv):
    import ctypes as C
    import torch
    p = workloads.uniform_cube(6000, seed=51)
    req = _run(srv, serve.Request.p3d(p, n_steps=2, dt=1e-3))
    rec = torch.from_numpy(serve.p3d_records(p)).cuda()
    vel = torch.empty((len(p), 3), dtype=torch.float32, device="cuda")
    dv = torch.empty_like(vel)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        assert gpu.lib.cvtx_gb300_dev_P3D_step(rec.data_ptr(), len(p), vel.data_ptr(),
                                               dv.data_ptr(), 1, SIG, 1e-3, stream) == 0
    assert gpu.lib.cvtx_gb300_dev_status(stream) == 0
    got = rec.cpu().numpy()
    # the device API plans its own split count, so agreement is to rounding
    assert exact.rel_l2(got, req.state_out) <= 1e-6
    assert exact.rel_l2(vel.cpu().numpy(), req.vel_out) <= TOL


def test_admission_waits_for_memory(gpu):
    """A budget that holds only a few requests at a time: the queue waits for
    memory, every request completes, and results equal those of a roomy
    server."""
    roomy = [serve.Request.p3d(workloads.uniform_cube(6000 + 500 * i, seed=60 + i), n_steps=2)
             for i in range(8)]
    tight = [serve.Request.p3d(workloads.uniform_cube(6000 + 500 * i, seed=60 + i), n_steps=2)
             for i in range(8)]
    with serve.Server(gpu.lib, n_slots=8, hbm_bytes=1 << 30) as s:
        for r in roomy:
            s.submit(r)
        assert s.drain(120_000)
    with serve.Server(gpu.lib, n_slots=8, hbm_bytes=1 << 20) as s:     # ~2 requests fit
        ids = [s.submit(r) for r in tight]
        assert s.drain(120_000)
        assert all(s.wait(i, 0) == 0 for i in ids)
        st = s.stats()
        assert st["completed"] == 8 and st["hbm_peak"] <= 1 << 20
    for a, b in zip(roomy, tight):
        assert np.array_equal(a.state_out, b.state_out)
