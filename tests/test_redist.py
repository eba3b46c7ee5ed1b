"""Particle redistribution on the host path (no accelerator enabled) against
the oracle's restatement of the reference algorithm: same count, same grid
points in the same (Morton) order, bit-identical strengths; plus the
properties the reference's scheme guarantees (total vorticity conserved by
the moment-preserving stencils, removal spreads the deficit). Parity with the
reference library itself is unpinned: its GCC build does not terminate in
these functions."""
import numpy as np
import pytest

from cvortex_gb300 import workloads
from oracle import redist as R
from redist_util import p2d, p3d

FUNCS = ("lambda0", "lambda1", "lambda2", "lambda3", "m4p")


@pytest.mark.parametrize("fname", FUNCS)
@pytest.mark.parametrize("neg, max_out", [(0.0, 10**6), (1e-2, 10**6), (0.1, 300)])
def test_p3d_host_matches_oracle(host, fname, neg, max_out):
    p = workloads.uniform_cube(700, seed=3)
    n, out = p3d(host.lib, p, fname, 0.2, neg, max_out)
    cnt, coord, vort = R.redistribute(p["coord"], p["vorticity"], fname, 0.2, neg, max_out)
    assert n == cnt
    assert np.array_equal(out["coord"], coord)
    assert np.array_equal(out["vorticity"], vort)
    assert np.all(out["volume"] == np.float32(0.2) ** 3)


@pytest.mark.parametrize("fname", FUNCS)
@pytest.mark.parametrize("neg, max_out", [(0.0, 10**6), (1e-2, 10**6), (0.05, 200)])
def test_p2d_host_matches_oracle(host, fname, neg, max_out):
    q = workloads.gaussian_patch_2d(900, seed=4)
    n, out = p2d(host.lib, q, fname, 0.05, neg, max_out)
    cnt, coord, vort = R.redistribute(q["coord"], q["vorticity"], fname, 0.05, neg, max_out)
    assert n == cnt
    assert np.array_equal(out["coord"], coord)
    assert np.array_equal(out["vorticity"], vort[:, 0])


@pytest.mark.parametrize("fname", ("lambda1", "lambda2", "lambda3", "m4p"))
def test_total_vorticity_conserved(host, fname):
    # stencils that reproduce constants keep the total; removal re-spreads it
    p = workloads.vortex_ring(2000, seed=5)
    for neg in (0.0, 0.05):
        n, out = p3d(host.lib, p, fname, 0.05, neg, 10**6)
        tot_in = p["vorticity"].astype(np.float64).sum(0)
        tot_out = out["vorticity"].astype(np.float64).sum(0)
        assert np.allclose(tot_out, tot_in, rtol=1e-4, atol=1e-4 * np.abs(tot_in).max())


def test_output_in_morton_order_and_on_grid(host):
    p = workloads.uniform_cube(300, seed=6)
    n, out = p3d(host.lib, p, "m4p", 0.25, 0.0, 10**6)
    corner = R._grid(p["coord"].astype(np.float32), "m4p", 0.25)[0].astype(np.float64)
    c = out["coord"].astype(np.float64)
    k = np.rint((c - corner) / 0.25).astype(np.int64)
    assert np.allclose((c - corner) / 0.25, k, atol=1e-3)
    code = R._morton(k)
    assert np.all(np.diff(code.astype(np.float64)) > 0)


def test_null_output_returns_count_and_edges(host):
    p = workloads.uniform_cube(200, seed=7)
    n_full, _ = p3d(host.lib, p, "lambda3", 0.2, 1e-3, 10**6)
    n_null, _ = p3d(host.lib, p, "lambda3", 0.2, 1e-3, 0, null_output=True)
    assert n_null == n_full
    assert p3d(host.lib, p[:0], "lambda3", 0.2, 0.0, 10)[0] == 0
    one = p[:1].copy()
    n1, o1 = p3d(host.lib, one, "lambda1", 0.2, 0.0, 100)
    assert 1 <= n1 <= 8
    assert np.allclose(o1["vorticity"].sum(0), one["vorticity"][0], rtol=1e-6)


def test_oracle_redistribution_functions():
    # the reference's functions at known points (src/RedistFunc.cpp:35-96)
    u = np.array([0.0, 0.25, 0.5, 1.0, 1.5, 2.0, 2.5], np.float32)
    assert np.allclose(R.redist_func("lambda1", u), [1, 0.75, 0.5, 0, 0, 0, 0])
    assert np.allclose(R.redist_func("m4p", u), [1, 0.8671875, 0.5625, 0, -0.0625, 0, 0])
    assert np.allclose(R.redist_func("lambda3", u), [1, 0.8203125, 0.5625, 0, -0.0625, 0, 0])
