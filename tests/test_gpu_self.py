"""Self-interaction form (each unordered pair once; csrc/sym.cuh with the
operations of csrc/p3d_sym.cu and csrc/p2d_sym.cu): the particles acting on
themselves through the device API and through the cvtx_ ABI (velocity at the
particles' own coordinates, stretching and viscous exchange with the pointer
array as its own target array), P3D and P2D, for every regularisation and
op, on ragged sizes, against the oracle on sampled targets and against the
ordered-pair kernels (forced through the tuning table, or given the targets
as a separate copy) on every target."""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import REGS
from cvortex_gb300 import abi, workloads
from oracle import exact
from parity import TOL, check

pytestmark = pytest.mark.gpu

OPS = {"vel": 1, "dvort": 2, "veldvort": 3}


def _records(p):
    r = np.zeros((len(p), 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7] = p["coord"], p["volume"], p["vorticity"]
    return r


def _dev(gpu, torch, rec, n, reg, ops):
    v = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    d = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert gpu.lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                          v.data_ptr() if ops & 1 else None,
                                          d.data_ptr() if ops & 2 else None,
                                          abi.REG_IDS[reg], 0.05, sh) == 0
    assert gpu.lib.cvtx_gb300_dev_status(sh) == 0
    return (v.cpu().numpy() if ops & 1 else None), (d.cpu().numpy() if ops & 2 else None)


@pytest.mark.parametrize("reg", REGS)
@pytest.mark.parametrize("n", [25_000, 33_001, 70_000])
def test_self_form_vs_oracle_and_ordered_pairs(gpu, reg, n):
    import torch
    p = workloads.vortex_ring(n, seed=71) if n == 70_000 else workloads.uniform_cube(n, seed=72)
    rec = torch.from_numpy(_records(p)).cuda()
    idx = np.sort(np.random.Generator(np.random.PCG64(73)).choice(n, 1024, replace=False))
    sub = p[idx].copy()
    ref_v = oracle.p3d_vel(p, sub["coord"], reg, 0.05)
    ref_d = oracle.p3d_dvort(p, sub, reg, 0.05)
    bucket = gpu.lib.cvtx_gb300_size_bucket(n)
    for name, ops in OPS.items():
        v, d = _dev(gpu, torch, rec, n, reg, ops)
        # the ordered-pair kernel: a tuned configuration switches the form off
        assert gpu.lib.cvtx_gb300_p3d_set_tuned(abi.REG_IDS[reg], ops, bucket, 2) == 0
        try:
            v2, d2 = _dev(gpu, torch, rec, n, reg, ops)
        finally:
            gpu.lib.cvtx_gb300_p3d_set_tuned(abi.REG_IDS[reg], ops, bucket, -1)
        if ops & 1:
            check(v[idx], ref_v, reg, sub["coord"], p["coord"], 0.05)
            assert exact.rel_l2(v, v2) <= TOL, (name, exact.rel_l2(v, v2))
        if ops & 2:
            check(d[idx], ref_d, reg, sub["coord"], p["coord"], 0.05)
            assert exact.rel_l2(d, d2) <= TOL, (name, exact.rel_l2(d, d2))


def test_self_form_through_the_abi(gpu):
    """cvtx_P3D_M2M_vel at the particles' own coordinates and
    cvtx_P3D_M2M_dvort with the pointer array as its own targets."""
    p = workloads.uniform_cube(50_000, seed=74)
    vel = gpu.p3d_vel(p, p["coord"].copy(), "winckelmans", 0.05)
    dv = gpu.p3d_dvort(p, p, "winckelmans", 0.05, same=True)
    idx = np.arange(0, len(p), 37)
    sub = p[idx].copy()
    check(vel[idx], oracle.p3d_vel(p, sub["coord"], "winckelmans", 0.05))
    check(dv[idx], oracle.p3d_dvort(p, sub, "winckelmans", 0.05))
    fv, fd = gpu.p3d_vel_dvort(p, "winckelmans", 0.05)
    assert exact.rel_l2(fv, vel) <= 1e-6 and exact.rel_l2(fd, dv) <= 1e-6


def test_self_form_coincident_particles(gpu):
    """Distinct particles at one position contribute nothing to each other
    (reference src/P3D.cpp:94-95) in the self-interaction form too."""
    p = workloads.uniform_cube(40_000, seed=75)
    p["coord"][20_000:20_100] = p["coord"][0]
    vel, dv = gpu.p3d_vel_dvort(p, "singular", 0.05)
    assert np.all(np.isfinite(vel)) and np.all(np.isfinite(dv))
    idx = np.concatenate([np.arange(0, 40_000, 97), [0, 20_000, 20_050]])
    sub = p[idx].copy()
    check(vel[idx], oracle.p3d_vel(p, sub["coord"], "singular", 0.05))
    check(dv[idx], oracle.p3d_dvort(p, sub, "singular", 0.05))


def _dev_visc(gpu, torch, rec, tgt, n, reg, nu):
    out = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert gpu.lib.cvtx_gb300_dev_P3D_M2M_visc(rec.data_ptr(), n, tgt.data_ptr(), 2, n,
                                               out.data_ptr(), abi.REG_IDS[reg], 0.05,
                                               C.c_float(nu), sh) == 0
    assert gpu.lib.cvtx_gb300_dev_status(sh) == 0
    return out.cpu().numpy()


@pytest.mark.parametrize("reg", ["winckelmans", "gaussian"])
@pytest.mark.parametrize("n", [33_001, 70_000])
def test_viscous_self_form_vs_oracle_and_ordered_pairs(gpu, reg, n):
    """The viscous exchange of the particles with themselves in the
    self-interaction form, against the oracle on sampled targets and against
    the ordered-pair kernel (targets passed as a separate copy of the
    records) on every target."""
    import torch
    nu = 1e-3
    p = workloads.vortex_ring(n, seed=76) if n == 70_000 else workloads.uniform_cube(n, seed=77)
    rec = torch.from_numpy(_records(p)).cuda()
    self_out = _dev_visc(gpu, torch, rec, rec, n, reg, nu)
    ordered = _dev_visc(gpu, torch, rec, rec.clone(), n, reg, nu)
    assert np.all(np.isfinite(self_out))
    assert exact.rel_l2(self_out, ordered) <= TOL, exact.rel_l2(self_out, ordered)
    idx = np.sort(np.random.Generator(np.random.PCG64(78)).choice(n, 1024, replace=False))
    sub = p[idx].copy()
    ref = oracle.p3d_visc(p, sub, reg, 0.05, nu)
    check(self_out[idx], ref, reg, sub["coord"], p["coord"], 0.05)
    # the cvtx_ ABI with the pointer array as its own targets takes the same form
    via_abi = gpu.p3d_visc(p, p, reg, 0.05, nu, same=True)
    assert exact.rel_l2(via_abi, self_out) <= 1e-6


def _records2d(q):
    return np.ascontiguousarray(
        np.stack([q["coord"][:, 0], q["coord"][:, 1], q["vorticity"], q["area"]], 1), np.float32)


def _dev_p2d(gpu, torch, rec, tgt, n, reg, nu=None):
    sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if nu is None:
        out = torch.full((n, 2), float("nan"), dtype=torch.float32, device="cuda")
        assert gpu.lib.cvtx_gb300_dev_P2D_M2M_vel(rec.data_ptr(), n, tgt.data_ptr(), n,
                                                  out.data_ptr(), abi.REG_IDS[reg], 0.05, sh) == 0
    else:
        out = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        assert gpu.lib.cvtx_gb300_dev_P2D_M2M_visc(rec.data_ptr(), n, tgt.data_ptr(), n,
                                                   out.data_ptr(), abi.REG_IDS[reg], 0.05,
                                                   C.c_float(nu), sh) == 0
    assert gpu.lib.cvtx_gb300_dev_status(sh) == 0
    return out.cpu().numpy()


@pytest.mark.parametrize("reg", REGS)
@pytest.mark.parametrize("n", [33_001, 70_000])
def test_p2d_velocity_self_form(gpu, reg, n):
    """P2D velocity at the particles' own positions in the self-interaction
    form, against the ordered-pair kernel (the points passed as a separate
    copy of the records) on every particle and the oracle on sampled ones."""
    import torch
    q = workloads.gaussian_patch_2d(n, seed=91 + n % 7)
    rec = torch.from_numpy(_records2d(q)).cuda()
    got = _dev_p2d(gpu, torch, rec, rec, n, reg)
    ordered = _dev_p2d(gpu, torch, rec, rec.clone(), n, reg)
    assert np.all(np.isfinite(got))
    assert exact.rel_l2(got, ordered) <= TOL, exact.rel_l2(got, ordered)
    idx = np.sort(np.random.Generator(np.random.PCG64(92)).choice(n, 1024, replace=False))
    ref = oracle.p2d_vel(q, q["coord"][idx], reg, 0.05)
    check(got[idx], ref, reg, q["coord"][idx], q["coord"], 0.05)


@pytest.mark.parametrize("reg", ["winckelmans", "gaussian"])
@pytest.mark.parametrize("n", [33_001, 70_000])
def test_p2d_viscous_self_form(gpu, reg, n):
    """P2D viscous exchange of the particles with themselves in the
    self-interaction form, against the ordered-pair kernel on every particle
    and, on sampled particles, against FP64: no less accurate than the
    reference formulation or the ordered-pair kernel."""
    import torch
    nu = 1e-3
    q = workloads.gaussian_patch_2d(n, seed=93 + n % 7)
    rec = torch.from_numpy(_records2d(q)).cuda()
    got = _dev_p2d(gpu, torch, rec, rec, n, reg, nu)
    ordered = _dev_p2d(gpu, torch, rec, rec.clone(), n, reg, nu)
    assert np.all(np.isfinite(got))
    # the exchange cancels to a small fraction of its terms (the reference
    # formulation is 2.6e-5 from FP64 on the 200k patch): two FP32 summation
    # orders differ by about 1e-5, a fault by far more
    assert exact.rel_l2(got, ordered) <= 5 * TOL, exact.rel_l2(got, ordered)
    idx = np.sort(np.random.Generator(np.random.PCG64(94)).choice(n, 1024, replace=False))
    fp64 = oracle.exact_p2d_visc(q, q[idx], reg, 0.05, nu)
    ref = oracle.p2d_visc(q, q[idx], reg, 0.05, nu)
    e_self, e_ord, e_ref = (exact.rel_l2(x, fp64) for x in (got[idx], ordered[idx], ref))
    assert e_self <= 1.5 * max(e_ref, e_ord, TOL), (e_self, e_ord, e_ref)


def test_p2d_self_form_through_the_abi(gpu):
    """cvtx_P2D_M2M_vel at the particles' own coordinates and
    cvtx_P2D_M2M_visc_dvort with the pointer array as its own targets take
    the self-interaction form: equal to the device calls in that form."""
    import torch
    n = 50_000
    q = workloads.gaussian_patch_2d(n, seed=95)
    rec = torch.from_numpy(_records2d(q)).cuda()
    vel = gpu.p2d_vel(q, q["coord"].copy(), "winckelmans", 0.05)
    visc = gpu.p2d_visc(q, q, "winckelmans", 0.05, 1e-3, same=True)
    assert exact.rel_l2(vel, _dev_p2d(gpu, torch, rec, rec, n, "winckelmans")) <= 1e-6
    assert exact.rel_l2(visc, _dev_p2d(gpu, torch, rec, rec, n, "winckelmans", 1e-3)) <= 1e-6
    idx = np.arange(0, n, 53)
    check(vel[idx], oracle.p2d_vel(q, q["coord"][idx], "winckelmans", 0.05))


def _dev_vort(gpu, torch, rec, tgt, n, reg):
    out = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert gpu.lib.cvtx_gb300_dev_P3D_M2M_vort(rec.data_ptr(), n, tgt.data_ptr(), 2, n,
                                               out.data_ptr(), abi.REG_IDS[reg], 0.05, sh) == 0
    assert gpu.lib.cvtx_gb300_dev_status(sh) == 0
    return out.cpu().numpy()


@pytest.mark.parametrize("reg", ["winckelmans", "planetary", "gaussian"])
@pytest.mark.parametrize("n", [33_001, 70_000])
def test_vorticity_field_self_form(gpu, reg, n):
    """The vorticity field at the particles' own positions (5 sigma box) in
    the self-interaction form, against the ordered-pair kernel on every
    particle and the oracle on sampled ones; through the cvtx_ ABI (points
    equal to the particles' coordinates, as the Pedrizzetti relaxation
    passes them) the same form serves the call."""
    import torch
    p = workloads.vortex_ring(n, seed=96) if n == 70_000 else workloads.uniform_cube(n, seed=97)
    rec = torch.from_numpy(_records(p)).cuda()
    got = _dev_vort(gpu, torch, rec, rec, n, reg)
    ordered = _dev_vort(gpu, torch, rec, rec.clone(), n, reg)
    assert np.all(np.isfinite(got))
    assert exact.rel_l2(got, ordered) <= TOL, exact.rel_l2(got, ordered)
    idx = np.sort(np.random.Generator(np.random.PCG64(98)).choice(n, 1024, replace=False))
    check(got[idx], oracle.p3d_vort(p, p["coord"][idx], reg, 0.05))
    via_abi = gpu.p3d_vort(p, p["coord"].copy(), reg, 0.05)
    assert exact.rel_l2(via_abi, got) <= 1e-6


FALLBACK_CHILD = r"""
import ctypes as C, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[2])
from cvortex_gb300 import abi, workloads
cv = abi.Cvtx(); cv.initialise()
lib = cv.lib
n = int(sys.argv[3])
p = workloads.uniform_cube(n, seed=99)
r = np.zeros((n, 8), np.float32)
r[:, 0:3], r[:, 3], r[:, 4:7] = p["coord"], p["volume"], p["vorticity"]
rec = torch.from_numpy(r).cuda()
sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
outs = []
for tgt in (rec, rec.clone()):          # the particles themselves, then a copy
    v = torch.full((n, 3), float("nan"), device="cuda")
    d = torch.full((n, 3), float("nan"), device="cuda")
    rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, tgt.data_ptr(), 2, n, v.data_ptr(),
                                    d.data_ptr(), 1, 0.05, sh)
    assert rc == 0 and lib.cvtx_gb300_dev_status(sh) == 0, cv.last_error()
    outs.append(np.concatenate([v.cpu().numpy(), d.cpu().numpy()], 1))
np.save(sys.argv[1], np.stack(outs))
"""


def _fallback_child(tmp_path, n, env):
    import os
    import subprocess
    import sys
    from pathlib import Path
    out = tmp_path / "fallback.npy"
    root = Path(__file__).resolve().parents[1]
    res = subprocess.run([sys.executable, "-c", FALLBACK_CHILD, str(out), str(root), str(n)],
                         cwd=root, env=dict(os.environ, **env), capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    return np.load(out)


def test_self_form_workspace_fallbacks(gpu, tmp_path):
    """The ordered-pair kernels serve a call that would take the
    self-interaction form (1) when the form's workspace cap leaves too few
    work items (CVTX_GB300_SYM_WS_CAP lowered), and (2) when its workspace
    cannot be allocated (CVTX_GB300_WS_LIMIT between the two forms'
    workspaces: an injected out-of-memory). Either way the call succeeds and
    equals the ordered-pair kernel on a copy of the particles bit for bit;
    with neither, the form is taken (results differ in rounding only)."""
    n = 40_000
    q = gpu.lib.cvtx_gb300_dev_P3D_M2M_ws_bytes
    ordered_ws, self_ws = q(n, n, 1, 1, 3, 0), q(n, n, 1, 1, 3, 1)
    assert 0 < ordered_ws < self_ws, (ordered_ws, self_ws)
    base = _fallback_child(tmp_path, n, {})
    assert not np.array_equal(base[0], base[1])
    assert exact.rel_l2(base[0], base[1]) <= TOL
    capped = _fallback_child(tmp_path, n, {"CVTX_GB300_SYM_WS_CAP": str(1 << 20)})
    assert np.array_equal(capped[0], capped[1])
    limit = (ordered_ws + self_ws) // 2
    limited = _fallback_child(tmp_path, n, {"CVTX_GB300_WS_LIMIT": str(limit)})
    assert np.array_equal(limited[0], limited[1])
    assert exact.rel_l2(limited[0], base[0]) <= TOL
