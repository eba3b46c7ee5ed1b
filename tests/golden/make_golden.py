"""Generate the golden fixtures in this directory from the reference library.

The reference CPU library is compiled from the reference sources by
oracle/build_ref.sh (into oracle/_ref/, not committed). This script feeds it
seeded inputs through the unchanged cvtx_ ABI (no accelerator: the
reference's OpenMP path) and stores inputs and outputs as compressed .npz:

* p3d_<set>.npz   -- vel / dvort / visc_dvort / vort for the four
                     regularisations on a uniform cube (700 particles,
                     sigma 0.2, plus 300 separate measurement points) and a
                     vortex ring (600 particles, sigma 0.05)
* p2d_patch.npz    -- P2D vel and visc_dvort for the four regularisations
* f3d_sheet.npz    -- F3D vel, dvort and influence matrix on a wake sheet
* reftest.npz      -- the reference's own CPU/GPU comparison tests
                     (reference test/testsamecpugpuresultsingle.h,
                     test/testsamecpugpuresultmany.h): the CPU result of every
                     section of all 10 repeats of both; the inputs come from
                     their LCG (tests/reftest_inputs.py), the first repeat's
                     are stored to pin it
* kat.npz          -- g, zeta, eta (3D and 2D) of every regularisation on a
                     grid of rho, from the reference's function pointers
* relax.npz        -- cvtx_P3D_pedrizzetti_relaxation of a vortex ring for
                     the four regularisations
* redist.npz       -- cvtx_P3D_redistribute_on_grid / cvtx_P2D_redistribute_on_grid
                     for the five redistribution functions with and without
                     removal of weak particles and with an output limit

Run from the repository root: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from cvortex_gb300 import abi, workloads  # noqa: E402

OUT = Path(__file__).resolve().parent
REGS = ("singular", "winckelmans", "planetary", "gaussian")
NU = 1e-3


def reference():
    oracle.build_ref()
    ref = oracle.ref_lib()
    if ref is None:
        raise SystemExit("reference library not available (oracle/build_ref.sh)")
    ref.initialise()
    assert ref.num_accelerators() == 0
    return ref


def p3d_case(ref, name, p, mes, sigma):
    d = {"particles": p, "mes": mes, "sigma": np.float32(sigma), "nu": np.float32(NU)}
    for reg in REGS:
        d[f"vel_{reg}"] = ref.p3d_vel(p, p["coord"], reg, sigma)
        d[f"velmes_{reg}"] = ref.p3d_vel(p, mes, reg, sigma)
        d[f"dvort_{reg}"] = ref.p3d_dvort(p, p, reg, sigma, same=True)
        d[f"visc_{reg}"] = ref.p3d_visc(p, p, reg, sigma, NU, same=True)
        d[f"vort_{reg}"] = ref.p3d_vort(p, mes, reg, sigma)
    np.savez_compressed(OUT / f"p3d_{name}.npz", **d)


def p2d_case(ref):
    q = workloads.gaussian_patch_2d(800)
    mes = q["coord"].copy()
    d = {"particles": q, "sigma": np.float32(0.05), "nu": np.float32(NU)}
    for reg in REGS:
        d[f"vel_{reg}"] = ref.p2d_vel(q, mes, reg, 0.05)
        d[f"visc_{reg}"] = ref.p2d_visc(q, q, reg, 0.05, NU, same=True)
    np.savez_compressed(OUT / "p2d_patch.npz", **d)


def f3d_case(ref):
    f = workloads.wake_sheet(500)
    t = workloads.sheet_targets(400)
    pts = workloads.uniform_cube(400, seed=77)
    pts["coord"] = t
    dirs = np.random.Generator(np.random.PCG64(78)).normal(size=(40, 3)).astype(np.float32)
    d = {"filaments": f, "mes": t, "particles": pts, "dirs": dirs,
         "vel": ref.f3d_vel(f, t), "dvort": ref.f3d_dvort(f, pts),
         "inf": ref.f3d_inf_mtrx(f[:200], t[:40], dirs)}
    np.savez_compressed(OUT / "f3d_sheet.npz", **d)


def reftest_case(ref):
    """The reference's own CPU-vs-GPU comparison tests, every section of all
    10 repeats of both (tests/reftest_inputs.py regenerates their inputs bit
    for bit from the test program's LCG), computed by the reference's CPU
    path. Key: <test>_r<repeat>_<section>."""
    sys.path.insert(0, str(ROOT / "tests"))
    import reftest_inputs as rt
    d = {"sigma": np.float32(rt.SIGMA), "nu": np.float32(rt.NU)}
    for test, k, a in rt.all_inputs():
        if k == 0:
            d[f"{test}_r0_p3"], d[f"{test}_r0_fil"], d[f"{test}_r0_p2"] = a["p3"], a["fil"], a["p2"]
        for key, op, reg in rt.SECTIONS:
            d[f"{test}_r{k}_{key}"] = rt.run_section(ref, op, reg, a)
    np.savez_compressed(OUT / "reftest.npz", **d)


def kat_case(ref):
    rho = np.concatenate([[0.0, 1e-4, 1e-3, 1e-2], np.linspace(0.05, 8.0, 160, dtype=np.float32)])
    rho = rho.astype(np.float32)
    d = {"rho": rho}
    for reg in REGS:
        vf = getattr(ref.lib, f"cvtx_VortFunc_{reg}")()
        d[f"g3_{reg}"] = np.array([vf.g_3D(float(r)) for r in rho], np.float32)
        d[f"g2_{reg}"] = np.array([vf.g_2D(float(r)) for r in rho], np.float32)
        d[f"zeta3_{reg}"] = np.array([vf.zeta_3D(float(r)) for r in rho], np.float32)
        if reg in ("winckelmans", "gaussian"):
            d[f"eta3_{reg}"] = np.array([vf.eta_3D(float(r)) for r in rho], np.float32)
            d[f"eta2_{reg}"] = np.array([vf.eta_2D(float(r)) for r in rho], np.float32)
        d[f"tag_{reg}"] = np.frombuffer(bytes(vf.cl_kernel_name_ext), np.uint8)
    np.savez_compressed(OUT / "kat.npz", **d)


REDIST_FUNCS = ("lambda0", "lambda1", "lambda2", "lambda3", "m4p")
# (negligible_vort, max_output_particles): keep all, remove weak ones,
# and an output limit that triggers the strength-threshold search
REDIST_P3D = ((0.0, 10**6), (1e-2, 10**6), (0.1, 150))
REDIST_P2D = ((0.0, 10**6), (1e-2, 10**6), (0.05, 100))


def redist_case(ref):
    sys.path.insert(0, str(ROOT / "tests"))
    from redist_util import p2d, p3d
    cube = workloads.uniform_cube(120, seed=21)
    ring = workloads.vortex_ring(100, seed=22)
    patch = workloads.gaussian_patch_2d(150, seed=23)
    one = abi.make_p3d([[0.013, 0.021, -0.007]], [[1.0, 0.5, -0.25]], [1.0])
    d = {"cube": cube, "ring": ring, "patch": patch, "one": one}

    def put(key, n, out):
        d[f"{key}_n"], d[f"{key}_coord"], d[f"{key}_vort"] = np.int64(n), out["coord"], out["vorticity"]

    for f in REDIST_FUNCS:
        for i, (neg, mo) in enumerate(REDIST_P3D):
            put(f"cube_{f}_{i}", *p3d(ref.lib, cube, f, 0.35, neg, mo))
        for i, (neg, mo) in enumerate(REDIST_P2D):
            put(f"patch_{f}_{i}", *p2d(ref.lib, patch, f, 0.1, neg, mo))
        put(f"one_{f}", *p3d(ref.lib, one, f, 0.1, 0.0, 1000))
    put("ring_m4p", *p3d(ref.lib, ring, "m4p", 0.15, 1e-3, 10**6))
    # edges: NULL output array (count only), empty input, and an output
    # limit whose threshold search removes every particle
    d["cube_m4p_null_n"] = np.int64(p3d(ref.lib, cube, "m4p", 0.35, 1e-2, 0, null_output=True)[0])
    d["empty_n"] = np.int64(p3d(ref.lib, cube[:0], "m4p", 0.35, 0.0, 10)[0])
    dense = workloads.gaussian_patch_2d(250, seed=23)
    d["dense"] = dense
    put("dense_lambda3", *p2d(ref.lib, dense, "lambda3", 0.05, 0.05, 100))
    np.savez_compressed(OUT / "redist.npz", **d)


def relax_case(ref):
    ring = workloads.vortex_ring(800, seed=31)
    d = {"particles": ring, "fdt": np.float32(0.3), "sigma": np.float32(0.05)}
    for reg in REGS:
        q = ring.copy()
        ref.relax(q, 0.3, reg, 0.05)
        d[f"vort_{reg}"] = q["vorticity"]
    np.savez_compressed(OUT / "relax.npz", **d)


def main():
    ref = reference()
    cube = workloads.uniform_cube(700, seed=11)
    mes = workloads.uniform_cube(300, seed=12)["coord"].copy()
    p3d_case(ref, "cube", cube, mes, 0.2)
    ring = workloads.vortex_ring(600, seed=13)
    p3d_case(ref, "ring", ring, workloads.vortex_ring(200, seed=14)["coord"].copy(), 0.05)
    p2d_case(ref)
    f3d_case(ref)
    reftest_case(ref)
    kat_case(ref)
    redist_case(ref)
    relax_case(ref)
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
