"""Particle redistribution: the oracle's restatement and the host path (no
accelerator enabled) against the reference library's own outputs (golden
fixture tests/golden/redist.npz, and the reference library live where it is
built), then the host path against the oracle (same count, same grid points
in the same Morton order, bit-identical strengths), plus the properties the
reference's scheme guarantees (total vorticity conserved by the
moment-preserving stencils, removal spreads the deficit).

Against the reference, counts and coordinates are bit-exact; strengths agree
to VORT_TOL of the largest strength, because the reference sums each grid
point in FP32 per OpenMP thread and the oracle in FP64 in particle order."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from cvortex_gb300 import workloads
from oracle import redist as R
from redist_util import p2d, p3d

FUNCS = ("lambda0", "lambda1", "lambda2", "lambda3", "m4p")
VORT_TOL = 2.0 ** -21
GOLD = np.load(Path(__file__).parent / "golden" / "redist.npz")
# (negligible_vort, max_output_particles) per case index, as the fixture
# generator (tests/golden/make_golden.py) uses them
GOLD_P3D = ((0.0, 10**6), (1e-2, 10**6), (0.1, 150))
GOLD_P2D = ((0.0, 10**6), (1e-2, 10**6), (0.05, 100))


def _gold_cases():
    """(key, dims, input, fname, gd, negligible, max_out) of every golden case."""
    out = []
    for f in FUNCS:
        for i, (neg, mo) in enumerate(GOLD_P3D):
            out.append((f"cube_{f}_{i}", 3, "cube", f, 0.35, neg, mo))
        for i, (neg, mo) in enumerate(GOLD_P2D):
            out.append((f"patch_{f}_{i}", 2, "patch", f, 0.1, neg, mo))
        out.append((f"one_{f}", 3, "one", f, 0.1, 0.0, 1000))
    out.append(("ring_m4p", 3, "ring", "m4p", 0.15, 1e-3, 10**6))
    out.append(("dense_lambda3", 2, "dense", "lambda3", 0.05, 0.05, 100))
    return out


GOLD_CASES = _gold_cases()


def assert_matches_gold(key, n, coord, vort):
    assert n == int(GOLD[f"{key}_n"])
    assert np.array_equal(coord, GOLD[f"{key}_coord"])
    if n == 0:
        return
    ref = GOLD[f"{key}_vort"].reshape(n, -1)
    vort = np.asarray(vort).reshape(n, -1)
    assert np.all(np.abs(vort - ref) <= VORT_TOL * np.abs(ref).max())


@pytest.mark.parametrize("case", GOLD_CASES, ids=[c[0] for c in GOLD_CASES])
def test_oracle_matches_reference_golden(case):
    key, dims, inp, fname, gd, neg, mo = case
    p = GOLD[inp]
    n, coord, vort = R.redistribute(p["coord"], p["vorticity"], fname, gd, neg, mo)
    assert_matches_gold(key, n, coord, vort)


@pytest.mark.parametrize("case", GOLD_CASES, ids=[c[0] for c in GOLD_CASES])
def test_host_matches_reference_golden(host, case):
    key, dims, inp, fname, gd, neg, mo = case
    call = p3d if dims == 3 else p2d
    n, out = call(host.lib, GOLD[inp], fname, gd, neg, mo)
    assert_matches_gold(key, n, out["coord"], out["vorticity"])


def test_reference_golden_edges(host):
    cube = GOLD["cube"]
    assert R.redistribute(cube["coord"], cube["vorticity"], "m4p", 0.35, 1e-2, None)[0] == \
        int(GOLD["cube_m4p_null_n"])
    assert p3d(host.lib, cube, "m4p", 0.35, 1e-2, 0, null_output=True)[0] == \
        int(GOLD["cube_m4p_null_n"])
    assert p3d(host.lib, cube[:0], "m4p", 0.35, 0.0, 10)[0] == int(GOLD["empty_n"]) == 0


@pytest.mark.parametrize("fname", FUNCS)
@pytest.mark.parametrize("dims", (2, 3))
def test_oracle_matches_reference_live(fname, dims):
    """Larger seeded sets than the fixture, against the reference library
    built from its sources (only where those sources are present)."""
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference library not built")
    if dims == 3:
        p, gd, neg, mo = workloads.uniform_cube(700, seed=3), 0.2, 0.1, 300
        n, out = p3d(ref.lib, p, fname, gd, neg, mo)
    else:
        p, gd, neg, mo = workloads.gaussian_patch_2d(900, seed=4), 0.05, 1e-2, 10**6
        n, out = p2d(ref.lib, p, fname, gd, neg, mo)
    cnt, coord, vort = R.redistribute(p["coord"], p["vorticity"], fname, gd, neg, mo)
    assert n == cnt
    assert np.array_equal(out["coord"], coord)
    ref_v = out["vorticity"].reshape(n, -1)
    assert np.all(np.abs(vort - ref_v) <= VORT_TOL * np.abs(ref_v).max())


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
