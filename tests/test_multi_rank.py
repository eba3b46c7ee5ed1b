"""The multi-rank path on CPU (gloo, world size 2): target sharding returns
exactly the single-process result, and the timing reduction takes the
slowest rank. Ranks call the library's host path (no accelerator enabled)."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from cvortex_gb300 import multi


def test_target_range_partitions():
    for n in (0, 1, 7, 100, 1001):
        for w in (1, 2, 3, 8):
            got = [multi.target_range(n, r, w) for r in range(w)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [h - l for l, h in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        multi.target_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, root, out_dir):
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    from cvortex_gb300 import abi, workloads
    from cvortex_gb300 import multi as m
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cv = abi.Cvtx()
        cv.initialise()
        cv.set_accelerated(False)
        p = workloads.uniform_cube(777, seed=9)
        vel, dv = m.sharded_p3d_vel_dvort(cv, p, "winckelmans", 0.05)
        slowest = m.max_over_ranks(float(rank + 1))
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), vel=vel, dv=dv, slowest=slowest)
    finally:
        dist.destroy_process_group()


def test_sharded_equals_single_process(built, cv, tmp_path):
    from conftest import ROOT
    from cvortex_gb300 import workloads
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(ROOT), str(tmp_path)),
                       nprocs=world, start_method="spawn", join=True)
    cv.set_accelerated(False)
    try:
        p = workloads.uniform_cube(777, seed=9)
        vel = cv.p3d_vel(p, p["coord"], "winckelmans", 0.05)
        dv = cv.p3d_dvort(p, p, "winckelmans", 0.05, same=True)
    finally:
        cv.set_accelerated(True)
    for r in range(world):
        d = np.load(tmp_path / f"r{r}.npz")
        assert np.array_equal(d["vel"], vel)
        assert np.array_equal(d["dv"], dv)
        assert float(d["slowest"]) == 2.0
