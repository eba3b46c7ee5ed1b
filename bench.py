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
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
# the serving measurement runs 32 slots, one hardware work queue each, so
# that no request's kernels queue behind another request's
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "P3D M2M vel+dvort Ginteractions/s"
UNIT = "Ginteractions/s"
# Canonical flops per interaction (add/sub/mul 1, FMA 2; special functions,
# compares and selects 0; per-call host constants excluded), by op and
# regularisation id (0 singular, 1 Winckelmans, 2 planetary, 3 Gaussian).
FLOPS = {("vel", 1): 30, ("dvort", 1): 46, ("veldvort", 1): 61,
         ("vel", 0): 25, ("dvort", 0): 39, ("veldvort", 0): 49,
         ("vel", 2): 25, ("dvort", 2): 39, ("veldvort", 2): 49,
         ("vel", 3): 46, ("dvort", 3): 62, ("veldvort", 3): 77}
# vorticity field (5 sigma box cut-off), FP32 operations per pair:
# winckelmans 22, planetary 15, gaussian 17
VORT_FLOPS = {1: 22, 2: 15, 3: 17}
REG = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}
OPS = {"veldvort": "fused vel+dvort", "vel": "vel", "dvort": "dvort",
       "vort": "vorticity field (5 sigma box cut-off)",
       "inf": "F3D influence matrix, 25,000 points x 20,000 filaments (2 GB)",
       "m2s": "few targets: fused vel+dvort of the first 64 particles from all sources",
       "f3d_dvort": "F3D vortex stretching, wake sheet of N filaments on N particles"}
M2S_TARGETS = 64
F3D_DVORT_FLOPS = 62
# influence matrix: F3D vel (51) + the dot with the direction (5) per entry
INF_FLOPS = 56
INF_SHAPE = (25_000, 20_000)
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
    ap.add_argument("--op", default="veldvort", choices=list(OPS),
                    help="the kernel timed as the step; the benchmark is veldvort, the others "
                         "exist to profile one kernel with the same command")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--serve-requests", type=int, default=64,
                    help="requests per arrival rate in the served-stream measurement")
    return ap.parse_args()


def profiled_traffic(n, reg):
    """DRAM bytes per launch of the benchmark kernel from the committed ncu
    summary (profiles/), when it covers this workload; else None."""
    if n != 100_000 or reg != "winckelmans":
        return None
    f = ROOT / "profiles" / "p3d_induce2_ring100k_launches.md"
    try:
        for line in f.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def dist_env():
    from cvortex_gb300.multi import dist_env as env
    return env()


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


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(p, reg, min_s=12.0, max_reps=40, sample=CPU_SAMPLE_TARGETS):
    """The reference CPU formulation on all host cores: vel + dvort for
    `sample` seeded targets against all sources, repeated until about `min_s`
    seconds of CPU work (at least three repeats)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_cores()))
    os.environ.setdefault("OMP_PROC_BIND", "spread")
    kind, ref = cpu_reference()
    idx = np.random.Generator(np.random.PCG64(7)).choice(len(p), min(sample, len(p)), replace=False)
    sub = p[np.sort(idx)].copy()
    cpu_step(kind, ref, p, sub[:64].copy(), reg)   # warm caches / thread pool
    t0 = time.perf_counter()
    reps = 0
    while reps < 3 or (time.perf_counter() - t0 < min_s and reps < max_reps):
        cpu_step(kind, ref, p, sub, reg)
        reps += 1
    dt = time.perf_counter() - t0
    pairs = reps * len(sub) * len(p)
    return {"value": pairs / dt / 1e9, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": kind, "cpu_model": cpu_model(), "omp_proc_bind": os.environ["OMP_PROC_BIND"],
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

    op = args.op
    if op == "vort" and reg not in VORT_FLOPS:
        raise SystemExit("--op vort: the singular vorticity field is zero (no kernel)")
    flops_per = (VORT_FLOPS[reg] if op == "vort" else INF_FLOPS if op == "inf"
                 else F3D_DVORT_FLOPS if op == "f3d_dvort"
                 else FLOPS[("veldvort", reg)] if op == "m2s" else FLOPS[(op, reg)])
    v_out = vel.data_ptr() if op in ("veldvort", "vel") else None
    d_out = dv.data_ptr() if op in ("veldvort", "dvort") else None
    pairs = float(n) * n
    if op == "m2s":
        pairs = float(n) * M2S_TARGETS
    if op == "inf":
        nm, ni = INF_SHAPE
        pairs = float(nm) * ni
        fil = workloads.wake_sheet(ni)
        rf = np.zeros((ni, 8), np.float32)
        rf[:, 0:3], rf[:, 3], rf[:, 4:7] = fil["start"], fil["strength"], fil["end"]
        tf = np.zeros((nm, 4), np.float32)
        tf[:, 0:3] = workloads.sheet_targets(nm)
        dirs = np.zeros((nm, 4), np.float32)
        dirs[:, 2] = 1.0
        rfd, tfd, dd = (torch.from_numpy(x).cuda() for x in (rf, tf, dirs))
        om = torch.empty((nm, ni), dtype=torch.float32, device="cuda")
    if op == "f3d_dvort":
        fil = workloads.wake_sheet(n)
        rf = np.zeros((n, 8), np.float32)
        rf[:, 0:3], rf[:, 3], rf[:, 4:7] = fil["start"], fil["strength"], fil["end"]
        rfd = torch.from_numpy(rf).cuda()
        rcube = torch.from_numpy(p3d_records(workloads.uniform_cube(n, seed=12)).reshape(n, 8)).cuda()

    def step():
        if op == "inf":
            rc = lib.cvtx_gb300_dev_F3D_inf_mtrx(rfd.data_ptr(), ni, tfd.data_ptr(), dd.data_ptr(),
                                                 nm, om.data_ptr(), sh)
        elif op == "m2s":
            rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, M2S_TARGETS,
                                            vel.data_ptr(), dv.data_ptr(), reg, SIGMA, sh)
        elif op == "f3d_dvort":
            rc = lib.cvtx_gb300_dev_F3D_M2M_dvort(rfd.data_ptr(), n, rcube.data_ptr(), 2, n,
                                                  vel.data_ptr(), sh)
        elif op == "vort":
            rc = lib.cvtx_gb300_dev_P3D_M2M_vort(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                 vel.data_ptr(), reg, SIGMA, sh)
        else:
            rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n, v_out, d_out,
                                            reg, SIGMA, sh)
        if rc != 0:
            raise RuntimeError(f"{op} step failed ({rc}): {cv.last_error()}")

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
    from cvortex_gb300.multi import max_over_ranks
    t_max = max_over_ranks(total_ms, device="cuda")
    value = world * args.steps * pairs / (t_max * 1e-3) / 1e9
    flops = flops_per * pairs
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": OPS[op] if op == "inf" else
                   OPS[op].replace("N ", f"{n} ") if op == "f3d_dvort" else
                   f"P3D vortex ring N={n}, {args.reg}, sigma={SIGMA}, {OPS[op]}"
                   + ("" if op == "m2s" else ", targets = sources"),
                   "interactions_per_step": pairs, "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None,
                     "traffic": profiled_traffic(n, args.reg) if op == "veldvort" else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "launch (profiles/p3d_induce2_ring100k_launches.md); "
                                       "algorithmic bytes 5.6 MB, the rest FP64 split partials",
                     "peak_source": "measured FP32 FMA probe, max of scalar FFMA "
                                    f"{p_scalar.value:.2f} and packed f32x2 FFMA "
                                    f"{p_packed.value:.2f} TFLOP/s",
                     "flops_per_interaction": flops_per,
                     "launch_ms": kernel_ms},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and not args.quick and op == "veldvort":
        out["e2e"] = e2e_abi(cv, p, args)
        out["serving"] = serve_extra(cv, lib, count=args.serve_requests)
        out["extras"] = extras(cv, lib, args, torch, sh, peak.value)
    if rank == 0 and world == 1 and op == "veldvort":
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


def measured_hbm_gbs():
    """Measured HBM copy bandwidth of this GPU model (MEASURED_PEAKS.json), or None."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return None


def extras(cv, lib, args, torch, sh, peak):
    """Per-op rates on the scale-up workloads and the 1M-particle target."""
    from cvortex_gb300 import workloads
    hbm_peak = measured_hbm_gbs()
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
            ms = timed_dev(f, torch, 5)
            row["visc"] = {"ginter_s": n * n / ms / 1e6,
                           "fp32_frac": (22 if r == 1 else 17) * n * n / (ms * 1e-3) / 1e12 / peak}
        if r in VORT_FLOPS:
            f = lambda: lib.cvtx_gb300_dev_P3D_M2M_vort(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                        o1.data_ptr(), r, SIGMA, sh)
            ms = timed_dev(f, torch, 5)
            row["vort"] = {"ginter_s": n * n / ms / 1e6,
                           "fp32_frac": VORT_FLOPS[r] * n * n / (ms * 1e-3) / 1e12 / peak}
        res[f"ring{n}_{rname}"] = row
    q = workloads.gaussian_patch_2d(200_000)
    rq = torch.from_numpy(np.ascontiguousarray(
        np.stack([q["coord"][:, 0], q["coord"][:, 1], q["vorticity"], q["area"]], 1))).cuda()
    o = torch.empty((len(q), 2), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_P2D_M2M_vel(rq.data_ptr(), len(q), rq.data_ptr(), len(q),
                                               o.data_ptr(), 3, SIGMA, sh)
    ms = timed_dev(f, torch, 5)
    res["p2d_patch200k_gaussian_vel"] = {"ginter_s": len(q) ** 2 / ms / 1e6,
                                         "fp32_frac": 13 * len(q) ** 2 / (ms * 1e-3) / 1e12 / peak}
    f = lambda: lib.cvtx_gb300_dev_P2D_M2M_vel(rq.data_ptr(), len(q), rq.data_ptr(), len(q),
                                               o.data_ptr(), 1, SIGMA, sh)
    ms = timed_dev(f, torch, 5)
    res["p2d_patch200k_winckelmans_vel"] = {"ginter_s": len(q) ** 2 / ms / 1e6,
                                            "fp32_frac": 15 * len(q) ** 2 / (ms * 1e-3) / 1e12 / peak}
    ov = torch.empty((len(q),), dtype=torch.float32, device="cuda")
    for rname, r, fl in (("winckelmans", 1, 16), ("gaussian", 3, 10)):
        f = lambda: lib.cvtx_gb300_dev_P2D_M2M_visc(rq.data_ptr(), len(q), rq.data_ptr(), len(q),
                                                    ov.data_ptr(), r, SIGMA, 1e-3, sh)
        ms = timed_dev(f, torch, 5)
        res[f"p2d_patch200k_{rname}_visc"] = {
            "ginter_s": len(q) ** 2 / ms / 1e6,
            "fp32_frac": fl * len(q) ** 2 / (ms * 1e-3) / 1e12 / peak}
    nf = 100_000
    fil = workloads.wake_sheet(nf)
    pts = workloads.sheet_targets(nf)
    rf = np.zeros((nf, 8), np.float32)
    rf[:, 0:3] = fil["start"]
    rf[:, 3] = fil["strength"]
    rf[:, 4:7] = fil["end"]
    tf = np.zeros((nf, 4), np.float32)
    tf[:, 0:3] = pts
    rfd, tfd = torch.from_numpy(rf).cuda(), torch.from_numpy(tf).cuda()
    of = torch.empty((nf, 3), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_F3D_M2M_vel(rfd.data_ptr(), nf, tfd.data_ptr(), 1, nf,
                                               of.data_ptr(), sh)
    ms = timed_dev(f, torch, 5)
    res["f3d_sheet100k_vel"] = {"ginter_s": nf * nf / ms / 1e6,
                                "fp32_frac": 51 * nf * nf / (ms * 1e-3) / 1e12 / peak}
    # influence matrix: write-bound (4 B per entry); 25,000 points x 20,000 filaments
    nm, ni = INF_SHAPE
    dirs = np.zeros((nm, 4), np.float32)
    dirs[:, 2] = 1.0
    dd = torch.from_numpy(dirs).cuda()
    om = torch.empty((nm, ni), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_F3D_inf_mtrx(rfd.data_ptr(), ni, tfd.data_ptr(), dd.data_ptr(),
                                                nm, om.data_ptr(), sh)
    ms = timed_dev(f, torch, 5)
    gbs = 4.0 * nm * ni / (ms * 1e-3) / 1e9
    res["f3d_inf_mtrx_25kx20k"] = {"ms": ms, "write_gbs": gbs,
                                   "hbm_frac": gbs / hbm_peak if hbm_peak else None,
                                   "hbm_peak_gbs": hbm_peak,
                                   "fp32_frac": INF_FLOPS * nm * ni / (ms * 1e-3) / 1e12 / peak}
    del om
    cube = workloads.uniform_cube(nf, seed=12)
    rc = torch.from_numpy(p3d_records(cube).reshape(nf, 8)).cuda()
    f = lambda: lib.cvtx_gb300_dev_F3D_M2M_dvort(rfd.data_ptr(), nf, rc.data_ptr(), 2, nf,
                                                 of.data_ptr(), sh)
    ms = timed_dev(f, torch, 3)
    res["f3d_sheet100k_dvort_cube100k"] = {"ginter_s": nf * nf / ms / 1e6,
                                           "fp32_frac": 62 * nf * nf / (ms * 1e-3) / 1e12 / peak}
    res["batch512"] = batch_extra(cv, lib, torch, sh)
    res["redistribute_ring200k_m4p"] = redistribute_extra(cv, lib)
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
    # the precision configuration's input: Gaussian, sigma 0.01, 1 % twins
    # closer than 1e-3 sigma (its errors against FP64 come from the tests)
    tw = workloads.cube_with_twins(m, 0.01)
    rb.copy_(torch.from_numpy(p3d_records(tw).reshape(m, 8)))
    f = lambda: lib.cvtx_gb300_dev_P3D_M2M(rb.data_ptr(), m, rb.data_ptr(), 2, m, b1.data_ptr(),
                                           b2.data_ptr(), 3, 0.01, sh)
    ms = timed_dev(f, torch, 2)
    res["twins1M_gaussian_veldvort"] = {
        "ginter_s": m * m / ms / 1e6, "ms": ms,
        "fp32_frac": FLOPS[("veldvort", 3)] * m * m / (ms * 1e-3) / 1e12 / peak}
    return res


def redistribute_extra(cv, lib, n=200_000, gd=0.01):
    """cvtx_P3D_redistribute_on_grid (M4' stencil, 125 grid points per
    particle) of a 200,000-particle vortex ring: the GPU path against this
    library's host path (all host cores); both give identical particles."""
    from cvortex_gb300 import abi, workloads
    p = workloads.vortex_ring(n)
    ptrs = abi.ptr_array(p)
    cap = 4 * n * 8
    out = np.zeros(cap, abi.P3D_DTYPE)
    rf = lib.cvtx_RedistFunc_m4p()

    def run():
        t0 = time.perf_counter()
        m = lib.cvtx_P3D_redistribute_on_grid(ptrs.ctypes.data, n, out.ctypes.data, cap,
                                              C.byref(rf), gd, 1e-3)
        return m, time.perf_counter() - t0

    run()
    m_gpu, t_gpu = min((run() for _ in range(3)), key=lambda x: x[1])
    cv.set_accelerated(False)
    try:
        m_host, t_host = run()
    finally:
        cv.set_accelerated(True)
    if m_gpu != m_host:
        raise RuntimeError("redistribution: GPU and host paths disagree")
    return {"particles_in": n, "particles_out": int(m_gpu), "grid_points_touched": n * 125,
            "gpu_ms": t_gpu * 1e3, "host_ms": t_host * 1e3, "host_cores": cpu_cores(),
            "speedup": t_host / t_gpu}


def batch_extra(cv, lib, torch, sh, count=512):
    """512 independent vel+dvort problems (uniform cube each, Winckelmans,
    sigma 0.05), sizes log-uniform in [1,000, 50,000]: one plain device call
    per problem vs the batched persistent launch (autotuned, graph-captured)."""
    from cvortex_gb300 import abi, workloads
    sizes = workloads.batch_sizes(count)
    keep, probs = [], []
    for i, n in enumerate(sizes):
        n = int(n)
        p = workloads.uniform_cube(n, seed=10_000 + i)
        rec = torch.from_numpy(p3d_records(p).reshape(n, 8)).cuda()
        v = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        d = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        keep.append((n, rec, v, d))
        probs.append(abi.cvtx_gb300_p3d_problem(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                v.data_ptr(), d.data_ptr(), SIGMA))
    pairs = float(sum(int(n) * int(n) for n in sizes))

    def plain():
        for n, rec, v, d in keep:
            rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n, v.data_ptr(),
                                            d.data_ptr(), 1, SIGMA, sh)
            if rc != 0:
                raise RuntimeError(cv.last_error())

    ms_plain = timed_dev(plain, torch, 2)

    def plain_separate():
        for n, rec, v, d in keep:
            for vel, dv in ((v, None), (None, d)):
                rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                vel.data_ptr() if vel is not None else None,
                                                dv.data_ptr() if dv is not None else None,
                                                1, SIGMA, sh)
                if rc != 0:
                    raise RuntimeError(cv.last_error())

    ms_plain_sep = timed_dev(plain_separate, torch, 2)
    arr = (abi.cvtx_gb300_p3d_problem * count)(*probs)
    b = lib.cvtx_gb300_batch_create(arr, count, 1, 3)
    if not b:
        raise RuntimeError(cv.last_error())
    try:
        t0 = time.perf_counter()
        if lib.cvtx_gb300_batch_tune(b, 1) != 0 or lib.cvtx_gb300_batch_capture(b) != 0:
            raise RuntimeError(cv.last_error())
        tune_s = time.perf_counter() - t0

        def batched():
            if lib.cvtx_gb300_batch_run(b, sh) != 0:
                raise RuntimeError(cv.last_error())

        ms_batch = timed_dev(batched, torch, 3)
        if lib.cvtx_gb300_batch_status(b) != 0:
            raise RuntimeError(cv.last_error())
        tpt, nt, chunk, items, graph = (C.c_int() for _ in range(5))
        lib.cvtx_gb300_batch_info(b, C.byref(tpt), C.byref(nt), C.byref(chunk), C.byref(items),
                                  C.byref(graph), None)
    finally:
        lib.cvtx_gb300_batch_destroy(b)
    return {"problems": count, "interactions": pairs,
            "sizes": [int(sizes.min()), int(sizes.max())],
            "plain_ms": ms_plain, "plain_ginter_s": pairs / ms_plain / 1e6,
            "plain_separate_ms": ms_plain_sep,
            "plain_separate_ginter_s": pairs / ms_plain_sep / 1e6,
            "plain_note": "plain = one fused vel+dvort device call per problem; plain_separate = "
                          "a vel call then a dvort call per problem",
            "batched_ms": ms_batch, "batched_ginter_s": pairs / ms_batch / 1e6,
            "speedup": ms_plain / ms_batch, "speedup_vs_separate": ms_plain_sep / ms_batch,
            "tuned_shape": [tpt.value, nt.value],
            "tuned_chunk": chunk.value, "items": items.value, "graph": bool(graph.value),
            "tune_s": tune_s}


SERVE_RATES = (100, 300, 1000, 3000, 5000)


def serve_extra(cv, lib, count=64, steps=10, dt=1e-3, rates=SERVE_RATES):
    """Served mixed-size stream vs plain per-request ABI calls.

    Stream: Poisson arrivals, 60% P3D vel+dvort (uniform cube, Winckelmans,
    sigma 0.05), 25% P2D vel (Gaussian patch, Winckelmans), 15% F3D vel (wake
    sheet on as many tracer points), sizes log-uniform on [500, 200,000],
    `steps` resident forward-Euler steps per client. The same requests are
    replayed at every rate (arrivals scale with 1/rate).

    served: the serving loop, latency = submit -> results in host memory.
    plain:  one request at a time through the reference ABI with host
            buffers (cvtx_P3D_M2M_vel + cvtx_P3D_M2M_dvort / cvtx_P2D_M2M_vel /
            cvtx_F3D_M2M_vel per step, Euler update on the host); its
            latencies at each rate are those of a FIFO queue fed the same
            arrivals, with each request's measured service time.
    """
    from cvortex_gb300 import serve, workloads
    arrival, kinds, sizes, seeds = workloads.serve_stream(count, rate=1.0)
    inputs = [workloads.serve_request_arrays(int(k), int(n), int(sd))
              for k, n, sd in zip(kinds, sizes, seeds)]

    def build():
        out = []
        for k, (a, b) in zip(kinds, inputs):
            kw = dict(n_steps=steps, dt=dt)
            out.append(serve.Request.p3d(a, **kw) if k == 0 else
                       serve.Request.p2d(a, **kw) if k == 1 else serve.Request.f3d(a, b, **kw))
        return out

    pairs = float(sum(r.interactions for r in build()))
    res = {"requests": count, "steps_per_client": steps,
           "mix": {"p3d_vel_dvort": int((kinds == 0).sum()), "p2d_vel": int((kinds == 1).sum()),
                   "f3d_vel": int((kinds == 2).sum())},
           "sizes": [int(sizes.min()), int(sizes.max())], "interactions": pairs, "rates": {}}
    srv = serve.Server(lib, n_slots=32)
    try:
        warm = build()[:4]                        # first-use costs out of the timed runs
        for r in warm:
            srv.submit(r)
        srv.drain()
        for rate in rates:
            srv.reset_stats()
            reqs = build()
            srv.replay(reqs, arrival / rate)
            if not srv.drain(600_000):
                raise RuntimeError("serving drain timed out")
            st = srv.stats()
            if st["completed"] != count:
                raise RuntimeError(f"served {st['completed']}/{count}: {cv.last_error()}")
            res["rates"][str(rate)] = {
                "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                "queue_p50_ms": st["queue_p50_ms"], "span_s": st["span_s"],
                "ginter_s": st["interactions"] / st["span_s"] / 1e9,
                "hbm_peak_bytes": st["hbm_peak"], "gpu_launches": st["kernel_launches"]}
    finally:
        srv.close()

    # plain per-request ABI calls, each request's service time measured once
    svc = []
    for k, (a, b) in zip(kinds, inputs):
        t0 = time.perf_counter()
        if k == 0:
            q = a.copy()
            for _ in range(steps):
                u = cv.p3d_vel(q, q["coord"], "winckelmans", SIGMA)
                w = cv.p3d_dvort(q, q, "winckelmans", SIGMA, same=True)
                q["coord"] += np.float32(dt) * u
                q["vorticity"] += np.float32(dt) * w
        elif k == 1:
            q = a.copy()
            for _ in range(steps):
                u = cv.p2d_vel(q, q["coord"], "winckelmans", SIGMA)
                q["coord"] += np.float32(dt) * u
        else:
            x = b.copy()
            for _ in range(steps):
                u = cv.f3d_vel(a, x)
                x += np.float32(dt) * u
        svc.append(time.perf_counter() - t0)
    if cv.last_error():
        raise RuntimeError(cv.last_error())
    svc = np.array(svc)
    plain = {"ginter_s_busy": pairs / svc.sum() / 1e9, "service_s_total": float(svc.sum()),
             "rates": {}}
    for rate in rates:
        arr = arrival / rate
        end, lat = 0.0, []
        for t, s in zip(arr, svc):
            end = max(end, t) + s
            lat.append(end - t)
        lat = np.array(lat) * 1e3
        plain["rates"][str(rate)] = {
            "p50_ms": float(np.percentile(lat, 50, method="inverted_cdf")),
            "p99_ms": float(np.percentile(lat, 99, method="inverted_cdf")),
            "ginter_s": pairs / (end - arr[0]) / 1e9}
    res["plain"] = plain
    res["speedup_ginter_s"] = {r: res["rates"][r]["ginter_s"] / plain["rates"][r]["ginter_s"]
                               for r in res["rates"]}
    return res


# ---- reference arm ---------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from cvortex_gb300 import workloads
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_cores()))
    os.environ.setdefault("OMP_PROC_BIND", "spread")
    kind, ref = cpu_reference()
    p = workloads.vortex_ring(args.n)
    order = np.random.Generator(np.random.PCG64(7)).permutation(args.n)
    # size each step's target sample so that all K steps take about a minute
    probe = p[np.sort(order[:128])].copy()
    for _ in range(max(args.warmup, 1)):
        t0 = time.perf_counter()
        cpu_step(kind, ref, p, probe, args.reg)
        per_target = (time.perf_counter() - t0) / len(probe)
    budget_s = 60.0
    m = int(budget_s / max(args.steps, 1) / max(per_target, 1e-9))
    m = max(64, min(CPU_SAMPLE_TARGETS, m, args.n))
    sub = p[np.sort(order[:m])].copy()
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
                            "cpu_model": cpu_model(),
                            "sample": f"each step: vel + dvort for {len(sub)} seeded targets x "
                                      f"{len(p)} sources (sample sized for about "
                                      f"{budget_s:.0f} s over {args.steps} steps)"},
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
