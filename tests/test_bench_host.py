"""Host-side logic of bench.py, the benchmark's one-line JSON contract: the
workload both arms name, the compact summary at the end of the line, and a
small run of the reference arm (the reference's CPU path on the host
cores; no GPU involved) checked key by key."""
import importlib.util
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_both_arms_name_the_same_workload():
    b = _bench()
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py"]
        args = b.parse()
    finally:
        sys.argv = sys_argv
    assert args.n == 1_000_000 and args.workload == "cube" and args.reg == "winckelmans"
    ours = b.workload_name(args, "veldvort")
    assert ours == b.workload_name(args)
    assert "N=1000000" in ours and "winckelmans" in ours and "vel + dvort" in ours


def test_summary_of_a_full_line():
    b = _bench()
    rate = {"served": [1.0, 2.0, 3.0], "plain": [4.0, 5.0, 6.0], "x": 1.5}
    ring = {k: {"ginter_s": v} for k, v in
            (("vel", 1.0), ("dvort", 2.0), ("veldvort", 3.0), ("visc", 4.0), ("vort", 5.0))}
    out = {"value": 967.01234, "roofline": {"frac": 0.74567}, "e2e": {"value": 842.4567},
           "extras": {"batch512": {"batched_ginter_s": 970.0, "speedup": 1.4,
                                   "speedup_vs_separate": 1.7},
                      "ring100k_winckelmans": ring,
                      "p2d_patch200k_winckelmans_vel": {"ginter_s": 10.0},
                      "p2d_patch200k_winckelmans_visc": {"ginter_s": 11.0},
                      "f3d_sheet100k_vel": {"ginter_s": 12.0},
                      "f3d_sheet100k_dvort_cube100k": {"ginter_s": 13.0}},
           "serving": {"light": {"rates": {"100": rate}}, "stream": {"rates": {"100": rate}}},
           "cpu_baseline": {"value": 0.3}}
    s = b.summary(out)
    assert s["value"] == 967.0 and s["fp32_frac"] == 0.7457 and s["e2e"] == 842.5
    assert s["batch512"] == [970.0, 1.4, 1.7]
    assert s["ring100k_w_vel_dvort_visc_vort"] == [1.0, 2.0, 4.0, 5.0]
    assert s["serving_light_p50_ms_served_plain"] == {"100": [1.0, 4.0]}
    assert s["serving_heavy_x"] == [1.5] and s["cpu_baseline"] == 0.3
    assert len(json.dumps(s)) < 600      # stays within the line's last characters


def test_reference_arm_line():
    """`bench.py --impl reference` on a small cube: one JSON line with the
    contract's keys, its e2e and cpu_baseline describing the same run."""
    oracle_lib = ROOT / "oracle" / "lib"
    if not oracle_lib.exists() or not any(oracle_lib.iterdir()):
        pytest.skip("oracle library not built")
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--n", "3000", "--steps", "2", "--warmup", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"]
    assert line["config"]["workload"].startswith("P3D uniform cube [-1,1]^3 N=3000")
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] == 2 and cb["kind"] in ("reference", "port")


def test_batch_op_takes_a_problem_count():
    """`--op batch` reads --n as a problem count; the default particle count
    would ask for a million problems and is refused before any CUDA call."""
    b = _bench()
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py", "--op", "batch", "--n", "128", "--quick"]
        args = b.parse()
        assert args.op == "batch" and args.n == 128
        assert b.OPS["batch"].replace("N ", "128 ").startswith("batch of 128 fused")
        sys.argv = ["bench.py", "--op", "batch"]
        with pytest.raises(SystemExit):
            b.parse()
    finally:
        sys.argv = sys_argv
    assert b.F3D_VEL_FLOPS == 51 and "f3d_vel" in b.OPS
