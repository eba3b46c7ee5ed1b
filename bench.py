#!/usr/bin/env python
"""Benchmark of the all-pairs P3D velocity + vortex-stretching path.

Workload (one "step"): velocity and stretching of every particle of a vortex
ring of 100,000 particles (radius 1, offsets N(0, 0.1^2), vorticity tangent
with magnitude exp(-d^2/(2 0.1^2)), Winckelmans regularisation, sigma 0.05),
i.e. 10^10 source-target interactions, each contributing to both outputs.
Inputs are seeded synthetic data (no dataset is involved).

Reported (one JSON line on rank 0):
  value      G interactions/s with the particle records resident in HBM
             (device-pointer API, fused vel+dvort kernel, caller's stream);
  e2e        the same metric through the reference C ABI with host buffers:
             cvtx_P3D_M2M_vel + cvtx_P3D_M2M_dvort per step, host gather,
             H2D and D2H inside the timed region;
  roofline   FP32-pipe roofline of the fused kernel: canonical flops per
             interaction (61 for Winckelmans vel+dvort) x interactions per
             launch / launch time, against the measured FP32 FMA peak;
  cpu_baseline  the reference CPU path (compiled reference library when it
             is loadable on this host, else the oracle's C restatement of it)
             on all host cores over a bounded sample of targets.
``--impl reference`` times that CPU implementation alone (the reference arm).
Multi-GPU (torchrun): every rank runs its own replica (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "P3D M2M vel+dvort Ginteractions/s"
UNIT = "Ginteractions/s"
# Canonical flops per interaction (add/sub/mul 1, FMA 2; special functions 0):
# Winckelmans vel 30, dvort 46, fused 61.
FLOPS = {("vel", 1): 30, ("dvort", 1): 46, ("veldvort", 1): 61,
         ("vel", 0): 25, ("dvort", 0): 39, ("veldvort", 0): 49,
         ("vel", 2): 25, ("dvort", 2): 39, ("veldvort", 2): 49,
         ("vel", 3): 46, ("dvort", 3): 62, ("veldvort", 3): 77}
REG = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}
SIGMA = 0.05
CPU_SAMPLE_TARGETS = 2048


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=100_000, help="particles in the ring")
    ap.add_argument("--reg", default="winckelmans", choices=list(REG))
    ap.add_argument("--quick", action="store_true", help="skip the extra measurements")
    ap.add_argument("--e2e-steps", type=int, default=5)
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def p3d_records(p):
    rec = np.zeros((len(p), 2, 4), np.float32)
    rec[:, 0, :3] = p["coord"]
    rec[:, 0, 3] = p["volume"]
    rec[:, 1, :3] = p["vorticity"]
    return rec


# ---- CPU implementation of the reference path --------------------------------
def cpu_reference():
    """(kind, handle): the compiled reference library when it loads on this
    host, else the oracle's restatement of the reference CPU path."""
    import oracle
    try:
        ref = oracle.ref_lib()
        if ref is not None:
            ref.initialise()
            return "reference", ref
    except OSError:
        pass
    oracle.build()
    return "port", None


def cpu_step(kind, ref, p, sub, reg):
    import oracle
    if kind == "reference":
        ref.p3d_vel(p, sub["coord"], reg, SIGMA)
        ref.p3d_dvort(p, sub, reg, SIGMA)
    else:
        oracle.p3d_vel(p, sub["coord"], reg, SIGMA)
        oracle.p3d_dvort(p, sub, reg, SIGMA)


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(p, reg, reps=3, sample=CPU_SAMPLE_TARGETS):
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_cores()))
    kind, ref = cpu_reference()
    idx = np.random.Generator(np.random.PCG64(7)).choice(len(p), min(sample, len(p)), replace=False)
    sub = p[np.sort(idx)].copy()
    cpu_step(kind, ref, p, sub[:64].copy(), reg)   # warm caches / thread pool
    t0 = time.perf_counter()
    for _ in range(reps):
        cpu_step(kind, ref, p, sub, reg)
    dt = time.perf_counter() - t0
    pairs = reps * len(sub) * len(p)
    return {"value": pairs / dt / 1e9, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": kind,
            "sample": f"{reps} x (vel + dvort) for {len(sub)} sampled targets x {len(p)} sources "
                      f"({dt:.1f} s of CPU time)"}


# ---- clocks ------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.lines, self.proc, self.gpu = [], None, gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "samples": len(sm),
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons)}


# ---- our arm -------------------------------------------------------------------
def run_ours(args):
    import torch
    from cvortex_gb300 import abi, workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cv = abi.Cvtx()
    cv.initialise()
    for i in range(cv.num_accelerators()):
        cv.lib.cvtx_accelerator_disable(i)
    cv.lib.cvtx_accelerator_enable(local)
    lib = cv.lib
    reg = REG[args.reg]
    n = args.n

    p = workloads.vortex_ring(n)
    rec = torch.from_numpy(p3d_records(p).reshape(n, 8)).cuda()
    vel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2
    stream = torch.cuda.current_stream()
    sh = C.c_void_p(stream.cuda_stream)

    def step():
        rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n, vel.data_ptr(),
                                        dv.data_ptr(), reg, SIGMA, sh)
        if rc != 0:
            raise RuntimeError(f"dev_P3D_M2M failed ({rc}): {cv.last_error()}")

    p_scalar, p_packed = C.c_double(0.0), C.c_double(0.0)
    if lib.cvtx_gb300_probe_fp32_detail(5, C.byref(p_scalar), C.byref(p_packed)) != 0:
        raise RuntimeError(cv.last_error())
    peak = C.c_double(max(p_scalar.value, p_packed.value))
    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        step()
    torch.cuda.synchronize()

    clocks = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = cv.launches()
    t_start.record()
    for k in range(args.steps):
        flush.zero_()            # L2 flush between steps (inputs are 3.2 MB)
        ev[k][0].record()
        step()
        ev[k][1].record()
    t_end.record()
    torch.cuda.synchronize()
    launches = cv.launches() - launches0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    kernel_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    t_max = total_ms
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t.item())
    pairs = float(n) * n
    value = world * args.steps * pairs / (t_max * 1e-3) / 1e9
    flops = FLOPS[("veldvort", reg)] * pairs
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"P3D vortex ring N={n}, {args.reg}, sigma={SIGMA}, "
                               "fused vel+dvort, targets = sources",
                   "interactions_per_step": pairs, "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None, "traffic": None,
                     "peak_source": "measured FP32 FMA probe, max of scalar FFMA "
                                    f"{p_scalar.value:.2f} and packed f32x2 FFMA "
                                    f"{p_packed.value:.2f} TFLOP/s",
                     "flops_per_interaction": FLOPS[("veldvort", reg)],
                     "launch_ms": kernel_ms},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and not args.quick:
        out["e2e"] = e2e_abi(cv, p, args)
        out["extras"] = extras(cv, lib, args, torch, sh, peak.value)
    if rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(p, args.reg)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def e2e_abi(cv, p, args):
    """Reference ABI with host buffers: cvtx_P3D_M2M_vel + cvtx_P3D_M2M_dvort."""
    from cvortex_gb300 import abi
    n = len(p)
    lib = cv.lib
    ptrs = abi.ptr_array(p)
    mes = np.ascontiguousarray(p["coord"])
    o1 = np.zeros((n, 3), np.float32)
    o2 = np.zeros((n, 3), np.float32)
    vf = C.byref(cv.vortfunc(args.reg))

    def call():
        lib.cvtx_P3D_M2M_vel(ptrs.ctypes.data, n, mes.ctypes.data, n, o1.ctypes.data, vf, SIGMA)
        lib.cvtx_P3D_M2M_dvort(ptrs.ctypes.data, n, ptrs.ctypes.data, n, o2.ctypes.data, vf, SIGMA)

    call()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        call()
    dt = (time.perf_counter() - t0) / args.e2e_steps
    if not (np.all(np.isfinite(o1)) and np.all(np.isfinite(o2))):
        raise RuntimeError(f"e2e produced non-finite results: {cv.last_error()}")
    vel_dv = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)

    def fused():
        rc = lib.cvtx_gb300_P3D_M2M_vel_dvort(ptrs.ctypes.data, n, vel_dv[0].ctypes.data,
                                              vel_dv[1].ctypes.data, vf, SIGMA)
        if rc != 0:
            raise RuntimeError(cv.last_error())

    fused()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        fused()
    dtf = (time.perf_counter() - t0) / args.e2e_steps
    return {"value": n * n / dt / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": n * (32 + 16) + n * 32,
            "d2h_bytes_per_step": 2 * (n * 12 + 4),
            "ms_per_step": dt * 1e3,
            "calls": "cvtx_P3D_M2M_vel + cvtx_P3D_M2M_dvort (reference ABI, host pointers)",
            "fused_extension": {"value": n * n / dtf / 1e9, "ms_per_step": dtf * 1e3,
                                "h2d_bytes_per_step": n * 32,
                                "d2h_bytes_per_step": 2 * n * 12 + 4,
                                "call": "cvtx_gb300_P3D_M2M_vel_dvort"}}


def timed_dev(fn, torch, reps):
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def extras(cv, lib, args, torch, sh, peak):
    """Per-op rates on the scale-up workloads and the 1M-particle target."""
    from cvortex_gb300 import workloads
    res = {}
    n = args.n
    p = workloads.vortex_ring(n)
    rec = torch.from_numpy(p3d_records(p).reshape(n, 8)).cuda()
    o1 = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    o2 = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    for rname, r in REG.items():
        row = {}
        for op, (a, b) in {"vel": (o1, None), "dvort": (None, o2), "veldvort": (o1, o2)}.items():
            f = lambda: lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                   a.data_ptr() if a is not None else None,
                                                   b.data_ptr() if b is not None else None,
                                                   r, SIGMA, sh)
            ms = timed_dev(f, torch, 5)
            row[op] = {"ginter_s": n * n / ms / 1e6,
                       "fp32_frac": FLOPS[(op, r)] * n * n / (ms * 1e-3) / 1e12 / peak}
        if r in (1, 3):
            f = lambda: lib.cvtx_gb300_dev_P3D_M2M_visc(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                        o1.data_ptr(), r, SIGMA, 1e-3, sh)
            row["visc"] = {"ginter_s": n * n / timed_dev(f, torch, 5) / 1e6}
        res[f"ring{n}_{rname}"] = row
    q = workloads.gaussian_patch_2d(200_000)
    rq = torch.from_numpy(np.ascontiguousarray(
        np.stack([q["coord"][:, 0], q["coord"][:, 1], q["vorticity"], q["area"]], 1))).cuda()
    o = torch.empty((len(q), 2), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_P2D_M2M_vel(rq.data_ptr(), len(q), rq.data_ptr(), len(q),
                                               o.data_ptr(), 3, SIGMA, sh)
    ms = timed_dev(f, torch, 5)
    res["p2d_patch200k_gaussian_vel"] = {"ginter_s": len(q) ** 2 / ms / 1e6}
    m = 1_000_000
    big = workloads.uniform_cube(m)
    rb = torch.from_numpy(p3d_records(big).reshape(m, 8)).cuda()
    b1 = torch.empty((m, 3), dtype=torch.float32, device="cuda")
    b2 = torch.empty((m, 3), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_P3D_M2M(rb.data_ptr(), m, rb.data_ptr(), 2, m, b1.data_ptr(),
                                           b2.data_ptr(), 1, SIGMA, sh)
    ms = timed_dev(f, torch, 2)
    res["cube1M_winckelmans_veldvort"] = {
        "ginter_s": m * m / ms / 1e6, "ms": ms,
        "fp32_frac": 61 * m * m / (ms * 1e-3) / 1e12 / peak}
    return res


# ---- reference arm ---------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from cvortex_gb300 import workloads
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_cores()))
    kind, ref = cpu_reference()
    p = workloads.vortex_ring(args.n)
    idx = np.random.Generator(np.random.PCG64(7)).choice(args.n, min(CPU_SAMPLE_TARGETS, args.n),
                                                         replace=False)
    sub = p[np.sort(idx)].copy()
    for _ in range(max(args.warmup, 1)):
        cpu_step(kind, ref, p, sub[:128].copy(), args.reg)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_step(kind, ref, p, sub, args.reg)
    dt = time.perf_counter() - t0
    pairs = args.steps * len(sub) * len(p)
    value = pairs / dt / 1e9
    cores = int(os.environ["OMP_NUM_THREADS"])
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": f"P3D vortex ring N={args.n}, {args.reg}, sigma={SIGMA}, "
                                  "vel + dvort, targets = sources",
                      "interactions_per_step": float(len(sub)) * len(p),
                      "parallelism": f"{cores} host threads (OpenMP)"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                            "sample": f"each step: vel + dvort for {len(sub)} sampled targets x "
                                      f"{len(p)} sources"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
