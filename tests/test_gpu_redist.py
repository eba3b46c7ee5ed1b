"""Particle redistribution on the GPU: the same grid points, order and
strengths as the host path and the oracle, bit for bit, and the reference
library's own outputs (golden fixture) to the FP32 summation tolerance."""
import numpy as np
import pytest

from cvortex_gb300 import workloads
from oracle import redist as R
from redist_util import p2d, p3d
from test_redist import GOLD, GOLD_CASES, assert_matches_gold

pytestmark = pytest.mark.gpu

FUNCS = ("lambda0", "lambda1", "lambda2", "lambda3", "m4p")


@pytest.mark.parametrize("fname", FUNCS)
@pytest.mark.parametrize("neg, max_out", [(0.0, 10**6), (1e-2, 10**6), (0.1, 300)])
def test_p3d_gpu_matches_oracle(gpu, fname, neg, max_out):
    p = workloads.uniform_cube(700, seed=3)
    launches = gpu.launches()
    n, out = p3d(gpu.lib, p, fname, 0.2, neg, max_out)
    assert gpu.launches() > launches, "redistribution did not run on the GPU"
    cnt, coord, vort = R.redistribute(p["coord"], p["vorticity"], fname, 0.2, neg, max_out)
    assert n == cnt
    assert np.array_equal(out["coord"], coord)
    assert np.array_equal(out["vorticity"], vort)


@pytest.mark.parametrize("case", GOLD_CASES, ids=[c[0] for c in GOLD_CASES])
def test_gpu_matches_reference_golden(gpu, case):
    key, dims, inp, fname, gd, neg, mo = case
    call = p3d if dims == 3 else p2d
    launches = gpu.launches()
    n, out = call(gpu.lib, GOLD[inp], fname, gd, neg, mo)
    assert gpu.launches() > launches, "redistribution did not run on the GPU"
    assert_matches_gold(key, n, out["coord"], out["vorticity"])


@pytest.mark.parametrize("fname", FUNCS)
def test_p2d_gpu_matches_oracle(gpu, fname):
    q = workloads.gaussian_patch_2d(900, seed=4)
    n, out = p2d(gpu.lib, q, fname, 0.05, 1e-2, 10**6)
    cnt, coord, vort = R.redistribute(q["coord"], q["vorticity"], fname, 0.05, 1e-2, 10**6)
    assert n == cnt
    assert np.array_equal(out["coord"], coord)
    assert np.array_equal(out["vorticity"], vort[:, 0])


def test_large_ring_gpu_equals_host(gpu):
    p = workloads.vortex_ring(100_000, seed=8)
    n_gpu, out_gpu = p3d(gpu.lib, p, "m4p", 0.02, 1e-3, 10**7)
    gpu.set_accelerated(False)
    try:
        n_host, out_host = p3d(gpu.lib, p, "m4p", 0.02, 1e-3, 10**7)
    finally:
        gpu.set_accelerated(True)
    assert n_gpu == n_host and n_gpu > 10_000
    assert np.array_equal(out_gpu["coord"], out_host["coord"])
    assert np.array_equal(out_gpu["vorticity"], out_host["vorticity"])
