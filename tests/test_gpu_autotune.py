"""The autotuner times every launch configuration, installs the fastest per
size bucket, and results stay within the parity bar whichever configuration
runs."""
import json

import numpy as np
import pytest

import oracle
from cvortex_gb300 import abi, autotune, workloads
from oracle import exact
from parity import TOL

pytestmark = pytest.mark.gpu


def test_tune_installs_and_keeps_parity(gpu, tmp_path):
    lib = gpu.lib
    res = autotune.tune(gpu, regs=("winckelmans",), ops=("veldvort",), sizes=(3000, 12000),
                        reps=1)
    assert len(res["entries"]) == 2
    for e in res["entries"]:
        assert lib.cvtx_gb300_p3d_current_config(1, 3, e["n"]) == e["best"]
        assert len(e["ms"]) == lib.cvtx_gb300_p3d_num_configs()
    path = autotune.save(res, tmp_path / "tuning.json")
    assert json.loads(path.read_text())[res["gpu"]]["entries"]
    p = workloads.uniform_cube(12000, seed=77)
    vel, dv = gpu.p3d_vel_dvort(p, "winckelmans", 0.05)
    idx = np.arange(0, len(p), 40)
    assert exact.rel_l2(vel[idx], oracle.p3d_vel(p, p["coord"][idx], "winckelmans", 0.05)) <= TOL
    # restore the built-in choice for the following tests
    for b in range(6):
        lib.cvtx_gb300_p3d_set_tuned(1, 3, b, -1)
    assert autotune.load(gpu, res["gpu"], path) == 2
    for b in range(6):
        lib.cvtx_gb300_p3d_set_tuned(1, 3, b, -1)


@pytest.mark.parametrize("cfg", range(11))
def test_every_configuration_matches_oracle(gpu, cfg):
    lib = gpu.lib
    n = 9000
    p = workloads.vortex_ring(n, seed=78)
    bucket = lib.cvtx_gb300_size_bucket(n)
    for reg in ("winckelmans", "gaussian"):
        rid = abi.REG_IDS[reg]
        lib.cvtx_gb300_p3d_set_tuned(rid, 3, bucket, cfg)
        try:
            vel, dv = gpu.p3d_vel_dvort(p, reg, 0.05)
        finally:
            lib.cvtx_gb300_p3d_set_tuned(rid, 3, bucket, -1)
        idx = np.arange(0, n, 30)
        v64, d64 = oracle.exact_p3d_vel_dvort(p, p["coord"][idx], p["vorticity"][idx], reg, 0.05)
        assert exact.rel_l2(vel[idx], v64) <= TOL, (reg, cfg)
        assert exact.rel_l2(dv[idx], d64) <= TOL, (reg, cfg)
