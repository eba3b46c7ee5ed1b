"""Autotuner for the P3D velocity / stretching kernels.

The library carries a table of launch configurations (targets per thread,
threads per CTA, packed two-wide FP32 or scalar arithmetic;
``cvtx_gb300_p3d_config_info``) and a tuning table that picks one per
(regularisation, ops, target-count bucket). ``tune`` times every
configuration on a representative problem of each requested size with the
device-pointer API and CUDA events, installs the fastest with
``cvtx_gb300_p3d_set_tuned`` and returns the measurements; ``save`` /
``load`` keep them in a JSON file keyed by GPU name so a later process can
install them without re-timing.
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from . import workloads
from .abi import REG_IDS

OPS = {"vel": 1, "dvort": 2, "veldvort": 3}
DEFAULT_CACHE = Path(__file__).resolve().parent / "lib" / "tuning.json"


def configs(lib) -> list[dict]:
    out = []
    for c in range(lib.cvtx_gb300_p3d_num_configs()):
        t, n, p = C.c_int(), C.c_int(), C.c_int()
        lib.cvtx_gb300_p3d_config_info(c, C.byref(t), C.byref(n), C.byref(p))
        out.append({"cfg": c, "tpt": t.value, "nt": n.value, "packed": bool(p.value)})
    return out


def _records(p):
    rec = np.zeros((len(p), 8), np.float32)
    rec[:, 0:3] = p["coord"]
    rec[:, 3] = p["volume"]
    rec[:, 4:7] = p["vorticity"]
    return rec


def time_config(lib, torch, rec, n, reg: int, ops: int, cfg: int, sigma: float, reps: int,
                vel, dv, stream) -> float:
    bucket = lib.cvtx_gb300_size_bucket(n)
    lib.cvtx_gb300_p3d_set_tuned(reg, ops, bucket, cfg)

    def call():
        rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                        vel.data_ptr() if ops & 1 else None,
                                        dv.data_ptr() if ops & 2 else None, reg, sigma, stream)
        if rc != 0:
            raise RuntimeError(f"dev_P3D_M2M failed ({rc})")

    call()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        call()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune(cv, regs=("winckelmans",), ops=("veldvort",), sizes=(3000, 20000, 100000, 400000),
         sigma: float = 0.05, reps: int = 3) -> dict:
    """Time every configuration; install the fastest per bucket."""
    import torch
    lib = cv.lib
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cfgs = configs(lib)
    result = {"gpu": torch.cuda.get_device_name(), "configs": cfgs, "entries": []}
    for n in sizes:
        p = workloads.vortex_ring(n, seed=1234)
        rec = torch.from_numpy(_records(p)).cuda()
        vel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        dv = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        bucket = lib.cvtx_gb300_size_bucket(n)
        for rname in regs:
            reg = REG_IDS[rname]
            for oname in ops:
                op = OPS[oname]
                times = {}
                for c in cfgs:
                    times[c["cfg"]] = time_config(lib, torch, rec, n, reg, op, c["cfg"], sigma,
                                                  reps, vel, dv, stream)
                best = min(times, key=times.get)
                lib.cvtx_gb300_p3d_set_tuned(reg, op, bucket, best)
                result["entries"].append({
                    "reg": rname, "ops": oname, "n": n, "bucket": bucket, "best": best,
                    "ms": {str(k): v for k, v in times.items()},
                    "ginter_s": n * n / times[best] / 1e6})
    return result


def save(result: dict, path: Path | str = DEFAULT_CACHE) -> Path:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    cache = json.loads(path.read_text()) if path.exists() else {}
    cache[result["gpu"]] = result
    path.write_text(json.dumps(cache, indent=1))
    return path


def load(cv, gpu_name: str, path: Path | str = DEFAULT_CACHE) -> int:
    """Install cached choices for this GPU; returns the number installed."""
    path = Path(path)
    if not path.exists():
        return 0
    res = json.loads(path.read_text()).get(gpu_name)
    if not res:
        return 0
    n = 0
    for e in res["entries"]:
        if cv.lib.cvtx_gb300_p3d_set_tuned(REG_IDS[e["reg"]], OPS[e["ops"]], e["bucket"],
                                           e["best"]) == 0:
            n += 1
    return n
