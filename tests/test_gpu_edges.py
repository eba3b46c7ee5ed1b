"""Edge cases of the CUDA path (through the C ABI) against the oracle:
empty and tiny sets, sizes around the tile boundaries, coincident points,
aliasing of sources and targets, few targets with many sources (source
splits) and the reverse, negative regularisation distance, filaments with
targets on their axis."""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import REGS
from cvortex_gb300 import abi, workloads
from oracle import exact
from parity import TOL, check

pytestmark = pytest.mark.gpu


def close(a, b, tol=1e-5):
    check(a, b, tol=tol)


def test_no_sources_gives_zeros(gpu):
    p = workloads.uniform_cube(1)
    mes = workloads.uniform_cube(300, seed=3)["coord"]
    out = np.full((300, 3), 5.0, np.float32)
    ptrs = abi.ptr_array(p)
    gpu.lib.cvtx_P3D_M2M_vel(ptrs.ctypes.data, 0, mes.ctypes.data, 300, out.ctypes.data,
                             C.byref(gpu.vortfunc("winckelmans")), 0.05)
    assert not np.any(out)


def test_no_sources_few_targets_gives_zeros(gpu):
    """Zero sources with a few targets (the few-target forms of every op):
    the outputs, prefilled, are overwritten with zeros."""
    lib, vf = gpu.lib, C.byref(gpu.vortfunc("winckelmans"))
    p = workloads.uniform_cube(5, seed=4)
    q = workloads.gaussian_patch_2d(5, seed=4)
    f = workloads.wake_sheet(3, seed=4)
    pp, qp, fp = abi.ptr_array(p), abi.ptr_array(q), abi.ptr_array(f)
    mes3 = np.ascontiguousarray(p["coord"])
    mes2 = np.ascontiguousarray(q["coord"])
    outs = [np.full((5, 3), 5.0, np.float32) for _ in range(4)] + [np.full((5, 2), 5.0, np.float32)]
    lib.cvtx_P3D_M2M_vel(pp.ctypes.data, 0, mes3.ctypes.data, 5, outs[0].ctypes.data, vf, 0.05)
    lib.cvtx_P3D_M2M_dvort(pp.ctypes.data, 0, pp.ctypes.data, 5, outs[1].ctypes.data, vf, 0.05)
    lib.cvtx_F3D_M2M_vel(fp.ctypes.data, 0, mes3.ctypes.data, 5, outs[2].ctypes.data)
    lib.cvtx_F3D_M2M_dvort(fp.ctypes.data, 0, pp.ctypes.data, 5, outs[3].ctypes.data)
    lib.cvtx_P2D_M2M_vel(qp.ctypes.data, 0, mes2.ctypes.data, 5, outs[4].ctypes.data, vf, 0.05)
    for o in outs:
        assert not np.any(o), o


@pytest.mark.parametrize("n", [1, 2, 31, 255, 256, 257, 511, 512, 513, 1023, 8191, 8192, 8193])
def test_sizes_around_tiles(gpu, n):
    p = workloads.uniform_cube(n, seed=n)
    vel, dv = gpu.p3d_vel_dvort(p, "winckelmans", 0.3)
    close(vel, oracle.p3d_vel(p, p["coord"], "winckelmans", 0.3))
    close(dv, oracle.p3d_dvort(p, p, "winckelmans", 0.3))


@pytest.mark.parametrize("reg", REGS)
def test_coincident_distinct_particles(gpu, reg):
    p = workloads.uniform_cube(600, seed=41)
    p["coord"][300:] = p["coord"][:300]          # 300 exact twins, different vorticity
    vel = gpu.p3d_vel(p, p["coord"], reg, 0.2)
    dv = gpu.p3d_dvort(p, p, reg, 0.2, same=True)
    x = p["coord"]
    ev, ed = exact.p3d_vel_dvort(p, x, p["vorticity"], reg, 0.2)
    check(vel, oracle.p3d_vel(p, x, reg, 0.2), reg, x, x, 0.2, ev)
    check(dv, oracle.p3d_dvort(p, p, reg, 0.2), reg, x, x, 0.2, ed)


def test_aliased_and_copied_targets_agree(gpu):
    p = workloads.vortex_ring(5000, seed=42)
    a = gpu.p3d_dvort(p, p, "gaussian", 0.05, same=True)
    b = gpu.p3d_dvort(p, p.copy(), "gaussian", 0.05)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("reg", REGS)
def test_few_targets_many_sources(gpu, reg):
    p = workloads.vortex_ring(60_000, seed=43)
    q = workloads.vortex_ring(3, seed=44)
    x, y = p["coord"], q["coord"]
    ev, ed = exact.p3d_vel_dvort(p, y, q["vorticity"], reg, 0.05)
    check(gpu.p3d_vel(p, y, reg, 0.05), oracle.p3d_vel(p, y, reg, 0.05), reg, y, x, 0.05, ev)
    check(gpu.p3d_dvort(p, q, reg, 0.05), oracle.p3d_dvort(p, q, reg, 0.05), reg, y, x, 0.05, ed)


@pytest.mark.parametrize("reg", REGS)
@pytest.mark.parametrize("n_tgt", [1, 5, 9, 100, 512])
def test_few_targets_every_op(gpu, reg, n_tgt):
    """The few-target kernel (sources spread over the threads, FP64
    shuffle reduction, fixed-order chunk sums): ragged target groups, a
    source count that does not fill its last chunk, targets on sources."""
    p = workloads.vortex_ring(200_003, seed=51)
    q = workloads.vortex_ring(n_tgt, seed=52)
    q["coord"][: min(2, n_tgt)] = p["coord"][:min(2, n_tgt)]
    x, y = p["coord"], q["coord"]
    ev, ed = oracle.exact_p3d_vel_dvort(p, y, q["vorticity"], reg, 0.05)
    check(gpu.p3d_vel(p, y, reg, 0.05), oracle.p3d_vel(p, y, reg, 0.05), reg, y, x, 0.05, ev)
    check(gpu.p3d_dvort(p, q, reg, 0.05), oracle.p3d_dvort(p, q, reg, 0.05), reg, y, x, 0.05, ed)


@pytest.mark.parametrize("n_tgt", [1, 7, 100])
def test_few_targets_p2d_f3d(gpu, n_tgt):
    """The few-target form of P2D velocity and F3D velocity and stretching:
    targets on sources, at filament ends and on a filament (the reference
    drops those terms)."""
    q = workloads.gaussian_patch_2d(300_001, seed=53)
    m = workloads.gaussian_patch_2d(n_tgt, seed=54)["coord"].copy()
    m[0] = q["coord"][0]
    for reg in REGS:
        close(gpu.p2d_vel(q, m, reg, 0.05), oracle.p2d_vel(q, m, reg, 0.05))
    f = workloads.wake_sheet(100_003, seed=55)
    t = workloads.sheet_targets(n_tgt, seed=56)
    t[0] = f["start"][5]
    if n_tgt > 2:
        t[1] = 0.5 * (f["start"][9] + f["end"][9])
    close(gpu.f3d_vel(f, t), oracle.f3d_vel(f, t))
    pts = workloads.uniform_cube(n_tgt, seed=57)
    pts["coord"] = t
    close(gpu.f3d_dvort(f, pts), oracle.f3d_dvort(f, pts))


def test_few_target_form_beyond_grid_limit(gpu):
    """The few-target form forced (tuning table) on 300,000 stretching
    targets: 75,000 groups of four, more than one grid dimension holds, so
    CTAs loop over target groups."""
    p = workloads.vortex_ring(3000, seed=57)
    q = workloads.uniform_cube(300_000, seed=58)
    lib = gpu.lib
    bucket = lib.cvtx_gb300_size_bucket(len(q))
    lib.cvtx_gb300_p3d_set_tuned(1, 2, bucket, 10)
    try:
        dv = gpu.p3d_dvort(p, q, "winckelmans", 0.05)
    finally:
        lib.cvtx_gb300_p3d_set_tuned(1, 2, bucket, -1)
    idx = np.r_[0:100, 150_000:150_100, 299_900:300_000]
    close(dv[idx], oracle.p3d_dvort(p, q[idx], "winckelmans", 0.05))


def test_many_targets_few_sources(gpu):
    p = workloads.uniform_cube(3, seed=45)
    mes = workloads.uniform_cube(40_000, seed=46)["coord"]
    close(gpu.p3d_vel(p, mes, "winckelmans", 0.05), oracle.p3d_vel(p, mes, "winckelmans", 0.05))


@pytest.mark.parametrize("reg", REGS)
def test_negative_sigma(gpu, reg):
    p = workloads.uniform_cube(700, seed=47)
    x = p["coord"]
    ev, ed = exact.p3d_vel_dvort(p, x, p["vorticity"], reg, -0.2)
    check(gpu.p3d_vel(p, x, reg, -0.2), oracle.p3d_vel(p, x, reg, -0.2), reg, x, x, -0.2, ev)
    check(gpu.p3d_dvort(p, p, reg, -0.2, same=True), oracle.p3d_dvort(p, p, reg, -0.2), reg, x, x,
          -0.2, ed)


def test_visc_without_eta_returns_zeros(gpu):
    p = workloads.uniform_cube(500, seed=48)
    for reg in ("singular", "planetary"):
        before = gpu.launches()
        out = gpu.p3d_visc(p, p, reg, 0.2, 1e-3, same=True)
        assert not np.any(out)
        assert gpu.launches() == before
    q = workloads.gaussian_patch_2d(500)
    for reg in ("singular", "planetary"):
        assert not np.any(gpu.p2d_visc(q, q, reg, 0.05, 1e-3, same=True))


def test_p2d_sizes_and_visc(gpu):
    for n in (1, 511, 512, 513, 9000):
        q = workloads.gaussian_patch_2d(n)
        close(gpu.p2d_vel(q, q["coord"], "winckelmans", 0.05),
              oracle.p2d_vel(q, q["coord"], "winckelmans", 0.05))
        for reg in ("winckelmans", "gaussian"):
            close(gpu.p2d_visc(q, q, reg, 0.05, 1e-3, same=True),
                  oracle.p2d_visc(q, q, reg, 0.05, 1e-3))


def test_f3d_targets_on_filament_axis(gpu):
    f = workloads.wake_sheet(300)
    t = workloads.sheet_targets(500)
    t[:50] = f["start"][:50]                       # exactly at segment ends
    t[50:100] = 0.5 * (f["start"][50:100] + f["end"][50:100])  # on the segment
    close(gpu.f3d_vel(f, t), oracle.f3d_vel(f, t))
    pts = workloads.uniform_cube(500, seed=49)
    pts["coord"] = t
    close(gpu.f3d_dvort(f, pts), oracle.f3d_dvort(f, pts))


def test_f3d_split_sources(gpu):
    f = workloads.wake_sheet(40_000)
    t = workloads.sheet_targets(50)
    close(gpu.f3d_vel(f, t), oracle.f3d_vel(f, t))


@pytest.mark.parametrize("reg", REGS)
def test_vort_and_relaxation(gpu, reg):
    p = workloads.vortex_ring(4000, seed=50)
    mes = p["coord"].copy()
    close(gpu.p3d_vort(p, mes, reg, 0.05), oracle.p3d_vort(p, mes, reg, 0.05))
    a = p.copy()
    b = p.copy()
    gpu.relax(a, 0.3, reg, 0.05)
    gpu.set_accelerated(False)
    gpu.relax(b, 0.3, reg, 0.05)
    gpu.set_accelerated(True)
    close(a["vorticity"], b["vorticity"], 1e-5)


def test_withheld_doorbell_reports_timeout(gpu):
    """A wait on an mbarrier that nothing completes runs out after its limit,
    the kernel records the expiry and returns, and the context keeps working."""
    import time
    t0 = time.perf_counter()
    assert gpu.lib.cvtx_gb300_selftest_withheld_wait(50.0) == 1
    assert time.perf_counter() - t0 < 5.0
    p = workloads.uniform_cube(500, seed=3)
    vel = gpu.p3d_vel(p, p["coord"], "winckelmans", 0.05)
    assert exact.rel_l2(vel, oracle.p3d_vel(p, p["coord"], "winckelmans", 0.05)) <= TOL


def test_dev_f3d_dvort_matches_oracle(gpu):
    import torch
    f = workloads.wake_sheet(3000, seed=5)
    p = workloads.uniform_cube(9000, seed=6)
    rf = np.zeros((len(f), 8), np.float32)
    rf[:, 0:3], rf[:, 3], rf[:, 4:7] = f["start"], f["strength"], f["end"]
    rp = np.zeros((len(p), 8), np.float32)
    rp[:, 0:3], rp[:, 3], rp[:, 4:7] = p["coord"], p["volume"], p["vorticity"]
    a, b = torch.from_numpy(rf).cuda(), torch.from_numpy(rp).cuda()
    out = torch.empty((len(p), 3), dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert gpu.lib.cvtx_gb300_dev_F3D_M2M_dvort(a.data_ptr(), len(f), b.data_ptr(), 2, len(p),
                                                out.data_ptr(), stream) == 0
    assert gpu.lib.cvtx_gb300_dev_status(stream) == 0
    close(out.cpu().numpy(), oracle.f3d_dvort(f, p))


def test_dev_p3d_vort_matches_abi(gpu):
    """The device-pointer vorticity field (point records, stride 1) equals the
    ABI call bit for bit."""
    import torch
    p = workloads.vortex_ring(5000, seed=17)
    mes = workloads.vortex_ring(9000, seed=18)["coord"].copy()
    rp = np.zeros((len(p), 8), np.float32)
    rp[:, 0:3], rp[:, 3], rp[:, 4:7] = p["coord"], p["volume"], p["vorticity"]
    rm = np.zeros((len(mes), 4), np.float32)
    rm[:, 0:3] = mes
    a, b = torch.from_numpy(rp).cuda(), torch.from_numpy(rm).cuda()
    out = torch.empty((len(mes), 3), dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for reg, code in (("winckelmans", 1), ("gaussian", 3), ("singular", 0)):
        out.fill_(7.0)
        assert gpu.lib.cvtx_gb300_dev_P3D_M2M_vort(a.data_ptr(), len(p), b.data_ptr(), 1,
                                                   len(mes), out.data_ptr(), code, 0.05,
                                                   stream) == 0
        assert gpu.lib.cvtx_gb300_dev_status(stream) == 0
        assert np.array_equal(out.cpu().numpy(), gpu.p3d_vort(p, mes, reg, 0.05))


@pytest.mark.parametrize("n", [8192, 8193, 20001])
def test_packed_p2d_f3d_ragged_sizes(gpu, n):
    """The packed P2D / F3D velocity kernels (8,192 targets and up) on sizes
    that do not fill the last target block, with coincident and on-axis
    targets."""
    q = workloads.gaussian_patch_2d(n, seed=9)
    idx = np.r_[0:64, n - 64:n]
    for reg in ("singular", "winckelmans", "gaussian", "planetary"):
        got = gpu.p2d_vel(q, q["coord"], reg, 0.05)
        close(got[idx], oracle.p2d_vel(q, q["coord"][idx], reg, 0.05))
    for reg in ("winckelmans", "gaussian"):
        got = gpu.p2d_visc(q, q, reg, 0.05, 1e-3, same=True)
        close(got[idx], oracle.p2d_visc(q, q[idx], reg, 0.05, 1e-3))
    f = workloads.wake_sheet(3000, seed=10)
    pts = workloads.sheet_targets(n, seed=11)
    pts[:40] = f["start"][:40]
    pts[40:80] = 0.5 * (f["start"][40:80] + f["end"][40:80])
    got = gpu.f3d_vel(f, pts)
    assert np.all(np.isfinite(got))
    sel = np.r_[0:128, n - 64:n]
    close(got[sel], oracle.f3d_vel(f, pts[sel]))


@pytest.mark.parametrize("n", [8192, 12001])
def test_packed_f3d_dvort(gpu, n):
    """The packed F3D stretching kernel (8,192 particles and up) against the
    oracle, with particles at filament ends (terms the reference drops) and
    zero-length filaments (whose per-filament 3 g / |r0| is infinite)."""
    f = workloads.wake_sheet(2000, seed=12)
    f["end"][[7, 300, 1999]] = f["start"][[7, 300, 1999]]
    p = workloads.uniform_cube(n, seed=13)
    p["coord"][:30] = f["start"][:30]
    p["coord"][30:60] = f["end"][30:60]
    got = gpu.f3d_dvort(f, p)
    assert np.all(np.isfinite(got))
    sel = np.r_[0:128, n - 64:n]
    close(got[sel], oracle.f3d_dvort(f, p[sel]))


@pytest.mark.parametrize("n", [8192, 8193, 12_345, 70_001])
def test_packed_p3d_vort_ragged_sizes(gpu, n):
    """The packed vorticity-field kernels (two targets per thread from 8,192
    targets, eight from 65,536) against the oracle on ragged sizes, with
    targets exactly on the 5 sigma box edge and on sources; one source split,
    and many splits (few sources)."""
    s = 0.05
    p = workloads.vortex_ring(3000, seed=15)
    mes = workloads.vortex_ring(n, seed=16)["coord"].copy()
    mes[:32] = p["coord"][:32]
    mes[32:64] = p["coord"][32:64] + np.float32(5 * s) * np.array([1, 0, 0], np.float32)
    idx = np.r_[0:128, n - 64:n]
    for reg in ("winckelmans", "planetary", "gaussian"):
        before = gpu.launches()
        got = gpu.p3d_vort(p, mes, reg, s)
        assert gpu.launches() > before
        close(got[idx], oracle.p3d_vort(p, mes[idx], reg, s))
        few = p[:40]
        close(gpu.p3d_vort(few, mes, reg, s)[idx], oracle.p3d_vort(few, mes[idx], reg, s))
    sing = gpu.p3d_vort(p, mes, "singular", s)
    assert not np.any(sing)


def test_dev_inf_mtrx_matches_abi(gpu):
    import torch
    f = workloads.wake_sheet(333, seed=14)
    pts = workloads.sheet_targets(257, seed=15)
    dirs = np.random.Generator(np.random.PCG64(16)).normal(size=(257, 3)).astype(np.float32)
    ref = gpu.f3d_inf_mtrx(f, pts, dirs)
    rf = np.zeros((len(f), 8), np.float32)
    rf[:, 0:3], rf[:, 3], rf[:, 4:7] = f["start"], f["strength"], f["end"]
    mp = np.zeros((257, 4), np.float32)
    mp[:, :3] = pts
    dp = np.zeros((257, 4), np.float32)
    dp[:, :3] = dirs
    a, m, d = (torch.from_numpy(x).cuda() for x in (rf, mp, dp))
    out = torch.empty((257, len(f)), dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert gpu.lib.cvtx_gb300_dev_F3D_inf_mtrx(a.data_ptr(), len(f), m.data_ptr(), d.data_ptr(),
                                               257, out.data_ptr(), stream) == 0
    assert gpu.lib.cvtx_gb300_dev_status(stream) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_device_call_then_abi_call_share_workspace(gpu):
    """A device-pointer call still running on a side stream, followed at once
    by a host-pointer ABI call: both use the context's split-sum workspace,
    so the second must wait for the first; both results match the oracle and
    each path's error word stays clean."""
    import torch
    p = workloads.uniform_cube(400_000, seed=61)
    rec = np.zeros((len(p), 8), np.float32)
    rec[:, 0:3], rec[:, 3], rec[:, 4:7] = p["coord"], p["volume"], p["vorticity"]
    drec = torch.from_numpy(rec).cuda()
    m = 6000                                   # split path: partials in the workspace
    vel = torch.empty((m, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((m, 3), dtype=torch.float32, device="cuda")
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    assert gpu.lib.cvtx_gb300_dev_P3D_M2M(drec.data_ptr(), len(p), drec.data_ptr(), 2, m,
                                          vel.data_ptr(), dv.data_ptr(), 1, 0.05,
                                          C.c_void_p(side.cuda_stream)) == 0
    q = workloads.vortex_ring(5000, seed=62)
    hv = gpu.p3d_vel(q, q["coord"], "winckelmans", 0.05)
    hd = gpu.p3d_dvort(q, q, "winckelmans", 0.05, same=True)
    assert gpu.lib.cvtx_gb300_dev_status(C.c_void_p(side.cuda_stream)) == 0
    check(hv, oracle.p3d_vel(q, q["coord"], "winckelmans", 0.05))
    check(hd, oracle.p3d_dvort(q, q, "winckelmans", 0.05))
    idx = np.arange(0, m, 7)
    sub = p[idx].copy()
    check(vel.cpu().numpy()[idx], oracle.p3d_vel(p, sub["coord"], "winckelmans", 0.05))
    check(dv.cpu().numpy()[idx], oracle.p3d_dvort(p, sub, "winckelmans", 0.05))
