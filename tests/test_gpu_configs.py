"""Every launch configuration that an environment variable can force (the
choices the built-in defaults pick by size), run on ragged sizes in a child
process each (the variables are read once per process), against the
oracle; the influence-matrix configurations must also agree bit for bit
(entries are independent, so only the CTA shape differs)."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from cvortex_gb300 import workloads
from parity import check

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[3])
from cvortex_gb300 import abi, workloads
from test_gpu_configs import problems
cv = abi.Cvtx(); cv.initialise()
assert cv.num_accelerators() > 0
before = cv.launches()
out = {k: v for k, v in problems(cv, sys.argv[2]).items()}
assert cv.launches() > before, "nothing ran on the GPU"
assert not cv.last_error(), cv.last_error()
np.savez(sys.argv[1], **out)
"""


def problems(cv, which):
    """The computations of one configuration family (used by the child)."""
    if which == "vort":
        p = workloads.vortex_ring(3000, seed=61)
        mes = workloads.vortex_ring(9001, seed=62)["coord"].copy()
        return {reg: cv.p3d_vort(p, mes, reg, 0.05)
                for reg in ("winckelmans", "planetary", "gaussian")}
    if which == "inf":
        out = {}
        for nf in (555, 556):     # ragged rows, and rows of whole float4 runs
            fil = workloads.wake_sheet(nf, seed=63)
            mes = workloads.sheet_targets(777, seed=64)
            dirs = np.random.Generator(np.random.PCG64(65)).normal(size=(777, 3))
            out[f"inf{nf}"] = cv.f3d_inf_mtrx(fil, mes, dirs.astype(np.float32))
        return out
    if which == "p2d":
        q = workloads.gaussian_patch_2d(9001, seed=66)
        return {"vel_w": cv.p2d_vel(q, q["coord"], "winckelmans", 0.05),
                "vel_g": cv.p2d_vel(q, q["coord"], "gaussian", 0.05),
                "visc_w": cv.p2d_visc(q, q, "winckelmans", 0.05, 1e-3, same=True),
                "visc_g": cv.p2d_visc(q, q, "gaussian", 0.05, 1e-3, same=True)}
    if which == "f3d":
        f = workloads.wake_sheet(3000, seed=67)
        return {"vel": cv.f3d_vel(f, workloads.sheet_targets(9001, seed=68))}
    if which == "f3d_dvort":
        f, pts = f3d_dvort_case()
        return {"dvort": cv.f3d_dvort(f, pts)}
    raise ValueError(which)


def f3d_dvort_case():
    """A wake sheet and 9,001 particles, some at filament ends."""
    f = workloads.wake_sheet(3000, seed=67)
    pts = workloads.uniform_cube(9001, seed=69)
    pts["coord"] = workloads.sheet_targets(9001, seed=68)
    pts["coord"][:20] = f["start"][:20]
    pts["coord"][4000:4020] = f["end"][40:60]
    return f, pts


def run_child(tmp_path, which, var, cfg):
    out = tmp_path / f"{which}_{cfg}.npz"
    env = dict(os.environ, **{var: str(cfg)})
    res = subprocess.run([sys.executable, "-c", CHILD, str(out), which, str(ROOT / "tests")],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    return dict(np.load(out))


# every target: a fault confined to one packed lane or one target slot of a
# thread would show on a fixed fraction of them
SAMPLE = slice(None)


@pytest.mark.parametrize("cfg", range(4))
def test_vort_configs(tmp_path, cfg):
    got = run_child(tmp_path, "vort", "CVTX_GB300_VORT_CFG", cfg)
    p = workloads.vortex_ring(3000, seed=61)
    mes = workloads.vortex_ring(9001, seed=62)["coord"].copy()
    for reg, v in got.items():
        check(v[SAMPLE], oracle.p3d_vort(p, mes[SAMPLE], reg, 0.05), tol=1e-5)


def test_inf_configs(tmp_path):
    runs = [run_child(tmp_path, "inf", "CVTX_GB300_INF_CFG", c) for c in range(6)]
    for nf in (555, 556):
        fil = workloads.wake_sheet(nf, seed=63)
        mes = workloads.sheet_targets(777, seed=64)
        dirs = np.random.Generator(np.random.PCG64(65)).normal(size=(777, 3)).astype(np.float32)
        check(runs[0][f"inf{nf}"], oracle.f3d_inf_mtrx(fil, mes, dirs), tol=1e-5)
        for r in runs[1:]:
            assert np.array_equal(r[f"inf{nf}"], runs[0][f"inf{nf}"])


@pytest.mark.parametrize("cfg", range(7))
def test_p2d_configs(tmp_path, cfg):
    got = run_child(tmp_path, "p2d", "CVTX_GB300_P2D_CFG", cfg)
    q = workloads.gaussian_patch_2d(9001, seed=66)
    check(got["vel_w"][SAMPLE], oracle.p2d_vel(q, q["coord"][SAMPLE], "winckelmans", 0.05), tol=1e-5)
    xy = q["coord"]
    check(got["vel_g"][SAMPLE], oracle.p2d_vel(q, q["coord"][SAMPLE], "gaussian", 0.05),
          "gaussian", xy[SAMPLE], xy, 0.05, tol=1e-5)
    check(got["visc_w"][SAMPLE], oracle.p2d_visc(q, q[SAMPLE], "winckelmans", 0.05, 1e-3), tol=1e-5)
    check(got["visc_g"][SAMPLE], oracle.p2d_visc(q, q[SAMPLE], "gaussian", 0.05, 1e-3),
          "gaussian", xy[SAMPLE], xy, 0.05, tol=1e-5)


@pytest.mark.parametrize("cfg", range(6))
def test_f3d_vel_configs(tmp_path, cfg):
    got = run_child(tmp_path, "f3d", "CVTX_GB300_F3D_CFG", cfg)
    f = workloads.wake_sheet(3000, seed=67)
    t = workloads.sheet_targets(9001, seed=68)
    check(got["vel"][SAMPLE], oracle.f3d_vel(f, t[SAMPLE]), tol=1e-5)


@pytest.mark.parametrize("cfg", range(5))
def test_f3d_dvort_configs(tmp_path, cfg):
    got = run_child(tmp_path, "f3d_dvort", "CVTX_GB300_F3D_DVORT_CFG", cfg)
    f, pts = f3d_dvort_case()
    check(got["dvort"][SAMPLE], oracle.f3d_dvort(f, pts[SAMPLE]), tol=1e-5)
