#!/usr/bin/env python
"""Benchmark of the all-pairs P3D velocity + vortex-stretching path.

Workload (one "step"): velocity and stretching of every particle of a
uniform cube of 1,000,000 particles (coordinates U[-1,1]^3, vorticity
components N(0, 0.1^2), volume 8/N, Winckelmans regularisation, sigma 0.05),
i.e. 10^12 source-target interactions, each contributing to both outputs.
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
  parity     the headline's results on sampled targets against the
             reference's CPU formulation (the oracle) and against FP64;
  extras     per-op rates of the scale-up, precision and batched workloads,
             each with its error against the FP64 oracle on sampled targets;
  serving    the served mixed-size stream against plain per-request calls
             (p50/p99 latency and interactions/s per arrival rate);
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
VISC_FLOPS = {1: 22, 3: 17}
# vorticity field (5 sigma box cut-off), FP32 operations per pair:
# winckelmans 22, planetary 15, gaussian 17
VORT_FLOPS = {1: 22, 2: 15, 3: 17}
REG = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}
REG_NAME = {v: k for k, v in REG.items()}
OPS = {"veldvort": "fused vel+dvort", "vel": "vel", "dvort": "dvort",
       "vort": "vorticity field (5 sigma box cut-off)",
       "inf": "F3D influence matrix, 25,000 points x 20,000 filaments (2 GB)",
       "m2s": "few targets: fused vel+dvort of the first 64 particles from all sources",
       "f3d_vel": "F3D velocity, wake sheet of N filaments at N points",
       "f3d_dvort": "F3D vortex stretching, wake sheet of N filaments on N particles",
       "batch": "batch of N fused vel+dvort problems, sizes log-uniform in [1,000, 50,000], "
                "winckelmans, sigma=0.05 (graph-captured persistent launches)",
       "visc": "P3D viscous exchange (nu 1e-3)",
       "p2d_vel": "P2D velocity, Gaussian vortex patch of N particles",
       "p2d_visc": "P2D viscous exchange (nu 1e-3), Gaussian vortex patch of N particles"}
P2D_FLOPS = {("vel", 0): 10, ("vel", 1): 15, ("vel", 2): 10, ("vel", 3): 13,
             ("visc", 1): 16, ("visc", 3): 10}
M2S_TARGETS = 64
F3D_VEL_FLOPS = 51
F3D_DVORT_FLOPS = 62
# influence matrix: F3D vel (51) + the dot with the direction (5) per entry
INF_FLOPS = 56
INF_SHAPE = (25_000, 20_000)
SIGMA = 0.05
CPU_SAMPLE_TARGETS = 1024
CHECK_TARGETS = 256          # sampled targets per FP64 / reference check


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cube", choices=["cube", "ring"],
                    help="cube: uniform cube (the plain workload's distribution); "
                         "ring: the scale-up vortex ring")
    ap.add_argument("--n", type=int, default=1_000_000,
                    help="particles (filaments for the F3D ops, problems for --op batch)")
    ap.add_argument("--reg", default="winckelmans", choices=list(REG))
    ap.add_argument("--quick", action="store_true", help="skip the extra measurements")
    ap.add_argument("--op", default="veldvort", choices=list(OPS),
                    help="the kernel timed as the step; the benchmark is veldvort, the others "
                         "exist to profile one kernel with the same command")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--serve-requests", type=int, default=64,
                    help="requests per arrival rate in the served-stream measurement")
    args = ap.parse_args()
    if args.op == "batch" and not 1 <= args.n <= 4096:
        ap.error("--op batch: --n is the number of problems, 1 to 4,096")
    return args


def dist_env():
    from cvortex_gb300.multi import dist_env as env
    return env()


def workload(args):
    from cvortex_gb300 import workloads
    if args.workload == "ring":
        return workloads.vortex_ring(args.n)
    return workloads.uniform_cube(args.n)


def workload_name(args, op="veldvort"):
    """The workload both arms name identically: velocity and stretching of
    every particle (the GPU arm runs them fused, the CPU arm as two calls)."""
    kind = ("P3D vortex ring" if args.workload == "ring" else
            "P3D uniform cube [-1,1]^3")
    what = "vel + dvort, targets = sources" if op == "veldvort" else OPS[op]
    return f"{kind} N={args.n}, {args.reg}, sigma={SIGMA}, {what}"


def p3d_records(p):
    rec = np.zeros((len(p), 2, 4), np.float32)
    rec[:, 0, :3] = p["coord"]
    rec[:, 0, 3] = p["volume"]
    rec[:, 1, :3] = p["vorticity"]
    return rec


def r4(x):
    """Four significant digits (keeps the JSON line short)."""
    return None if x is None else float(f"{x:.4g}")


def sample_idx(n, m=CHECK_TARGETS, seed=11):
    return np.sort(np.random.Generator(np.random.PCG64(seed)).choice(n, min(m, n), replace=False))


def errs(got, ref):
    """rel L2 and max per-target relative error of `got` against `ref`."""
    from oracle import exact
    return {"rel_l2": r4(exact.rel_l2(got, ref)), "max_rel": r4(exact.max_rel(got, ref))}


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
    seconds of CPU work (at least two repeats)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_cores()))
    os.environ.setdefault("OMP_PROC_BIND", "spread")
    kind, ref = cpu_reference()
    idx = np.random.Generator(np.random.PCG64(7)).choice(len(p), min(sample, len(p)), replace=False)
    sub = p[np.sort(idx)].copy()
    cpu_step(kind, ref, p, sub[:32].copy(), reg)   # warm caches / thread pool
    t0 = time.perf_counter()
    reps = 0
    while reps < 2 or (time.perf_counter() - t0 < min_s and reps < max_reps):
        cpu_step(kind, ref, p, sub, reg)
        reps += 1
    dt = time.perf_counter() - t0
    pairs = reps * len(sub) * len(p)
    return {"value": r4(pairs / dt / 1e9), "unit": UNIT,
            "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": kind,
            "cpu_model": cpu_model(), "omp_proc_bind": os.environ["OMP_PROC_BIND"],
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

    p = workload(args)
    rec = torch.from_numpy(p3d_records(p).reshape(n, 8)).cuda()
    vel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2
    stream = torch.cuda.current_stream()
    sh = C.c_void_p(stream.cuda_stream)

    op = args.op
    if op == "vort" and reg not in VORT_FLOPS:
        raise SystemExit("--op vort: the singular vorticity field is zero (no kernel)")
    if op in ("visc", "p2d_visc") and reg not in VISC_FLOPS:
        raise SystemExit(f"--op {op}: only winckelmans and gaussian have a viscous kernel")
    if op == "batch" and reg != REG["winckelmans"]:
        raise SystemExit("--op batch: the batch workload is winckelmans")
    flops_per = (VORT_FLOPS[reg] if op == "vort" else INF_FLOPS if op == "inf"
                 else F3D_DVORT_FLOPS if op == "f3d_dvort" else F3D_VEL_FLOPS if op == "f3d_vel"
                 else VISC_FLOPS[reg] if op == "visc"
                 else P2D_FLOPS[("vel", reg)] if op == "p2d_vel"
                 else P2D_FLOPS[("visc", reg)] if op == "p2d_visc"
                 else FLOPS[("veldvort", reg)] if op in ("m2s", "batch") else FLOPS[(op, reg)])
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
    if op in ("p2d_vel", "p2d_visc"):
        q = workloads.gaussian_patch_2d(n)
        rq = torch.from_numpy(np.ascontiguousarray(
            np.stack([q["coord"][:, 0], q["coord"][:, 1], q["vorticity"], q["area"]], 1))).cuda()
    if op in ("f3d_vel", "f3d_dvort"):
        fil = workloads.wake_sheet(n)
        rf = np.zeros((n, 8), np.float32)
        rf[:, 0:3], rf[:, 3], rf[:, 4:7] = fil["start"], fil["strength"], fil["end"]
        rfd = torch.from_numpy(rf).cuda()
    if op == "f3d_vel":
        tf = np.zeros((n, 4), np.float32)
        tf[:, 0:3] = workloads.sheet_targets(n)
        tfd = torch.from_numpy(tf).cuda()
    if op == "f3d_dvort":
        rcube = torch.from_numpy(p3d_records(workloads.uniform_cube(n, seed=12)).reshape(n, 8)).cuda()
    if op == "batch":
        bsizes = workloads.batch_sizes(n)
        pairs = float(sum(int(m) * int(m) for m in bsizes))
        bkeep, bprobs = [], []
        for i, m in enumerate(bsizes):
            m = int(m)
            brec = torch.from_numpy(
                p3d_records(workloads.uniform_cube(m, seed=10_000 + i)).reshape(m, 8)).cuda()
            bv = torch.empty((m, 3), dtype=torch.float32, device="cuda")
            bd = torch.empty((m, 3), dtype=torch.float32, device="cuda")
            bkeep.append((brec, bv, bd))
            bprobs.append(abi.cvtx_gb300_p3d_problem(brec.data_ptr(), m, brec.data_ptr(), 2, m,
                                                     bv.data_ptr(), bd.data_ptr(), SIGMA))
        barr = (abi.cvtx_gb300_p3d_problem * n)(*bprobs)
        bh = lib.cvtx_gb300_batch_create(barr, n, 1, 3)
        if not bh or lib.cvtx_gb300_batch_tune(bh, 1) != 0 or lib.cvtx_gb300_batch_capture(bh) != 0:
            raise RuntimeError(cv.last_error())

    def step():
        if op == "inf":
            rc = lib.cvtx_gb300_dev_F3D_inf_mtrx(rfd.data_ptr(), ni, tfd.data_ptr(), dd.data_ptr(),
                                                 nm, om.data_ptr(), sh)
        elif op == "m2s":
            rc = lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, M2S_TARGETS,
                                            vel.data_ptr(), dv.data_ptr(), reg, SIGMA, sh)
        elif op == "f3d_vel":
            rc = lib.cvtx_gb300_dev_F3D_M2M_vel(rfd.data_ptr(), n, tfd.data_ptr(), 1, n,
                                                vel.data_ptr(), sh)
        elif op == "batch":
            rc = lib.cvtx_gb300_batch_run(bh, sh)
        elif op == "f3d_dvort":
            rc = lib.cvtx_gb300_dev_F3D_M2M_dvort(rfd.data_ptr(), n, rcube.data_ptr(), 2, n,
                                                  vel.data_ptr(), sh)
        elif op == "vort":
            rc = lib.cvtx_gb300_dev_P3D_M2M_vort(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                 vel.data_ptr(), reg, SIGMA, sh)
        elif op == "visc":
            rc = lib.cvtx_gb300_dev_P3D_M2M_visc(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                 vel.data_ptr(), reg, SIGMA, 1e-3, sh)
        elif op == "p2d_vel":
            rc = lib.cvtx_gb300_dev_P2D_M2M_vel(rq.data_ptr(), n, rq.data_ptr(), n, vel.data_ptr(),
                                                reg, SIGMA, sh)
        elif op == "p2d_visc":
            rc = lib.cvtx_gb300_dev_P2D_M2M_visc(rq.data_ptr(), n, rq.data_ptr(), n, vel.data_ptr(),
                                                 reg, SIGMA, 1e-3, sh)
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
        flush.zero_()            # L2 flush between steps (inputs are 32 MB)
        ev[k][0].record()
        step()
        ev[k][1].record()
    t_end.record()
    torch.cuda.synchronize()
    launches = cv.launches() - launches0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    if op == "batch":
        bst = lib.cvtx_gb300_batch_status(bh)
        lib.cvtx_gb300_batch_destroy(bh)
        if bst != 0:
            raise RuntimeError(f"batch status {bst}: {cv.last_error()}")
    total_ms = t_start.elapsed_time(t_end)
    kernel_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    from cvortex_gb300.multi import max_over_ranks
    t_max = max_over_ranks(total_ms, device="cuda")
    value = world * args.steps * pairs / (t_max * 1e-3) / 1e9
    flops = flops_per * pairs
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    if op == "inf":
        wl = OPS[op]
    elif op in ("f3d_vel", "f3d_dvort", "batch"):
        wl = OPS[op].replace("N ", f"{n} ")
    elif op in ("p2d_vel", "p2d_visc"):
        wl = OPS[op].replace("N ", f"{n} ") + f", {args.reg}, sigma={SIGMA}"
    else:
        wl = workload_name(args, op) + ("" if op in ("m2s", "veldvort") else ", targets = sources")
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": wl, "interactions_per_step": pairs,
                   "kernel": "fused vel+dvort (device-pointer API)" if op == "veldvort" else op,
                   "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None,
                     "traffic": None,
                     "traffic_note": "not measured in this run (ncu summaries under profiles/); "
                                     "algorithmic bytes per launch 32 B x N in, 24 B x N out",
                     "peak_source": "measured FP32 FMA probe, max of scalar FFMA "
                                    f"{p_scalar.value:.2f} and packed f32x2 FFMA "
                                    f"{p_packed.value:.2f} TFLOP/s",
                     "flops_per_interaction": flops_per,
                     "launch_ms": kernel_ms},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and op == "veldvort":
        out["parity"] = headline_parity(p, vel, dv, args)
    if rank == 0 and not args.quick and op == "veldvort":
        out["e2e"] = e2e_abi(cv, p, args)
        out["extras"] = extras(cv, lib, args, torch, sh, peak.value)
        out["serving"] = serve_extra(cv, lib, count=args.serve_requests)
    if rank == 0 and world == 1 and op == "veldvort":
        out["cpu_baseline"] = cpu_baseline(p, args.reg)
    if rank == 0 and "extras" in out:
        out["summary"] = summary(out)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def summary(out):
    """The figures a reader of the line's last characters looks for, in
    short form (G interactions/s unless named otherwise)."""
    x, sv = out["extras"], out["serving"]
    b = x["batch512"]
    heavy = sv["stream"]["rates"]
    light = sv["light"]["rates"]
    return {
        "value": r4(out["value"]), "fp32_frac": r4(out["roofline"]["frac"]),
        "e2e": r4(out["e2e"]["value"]),
        "batch512": [b["batched_ginter_s"], b["speedup"], b["speedup_vs_separate"]],
        "ring100k_w_vel_dvort_visc_vort": [x["ring100k_winckelmans"][k]["ginter_s"]
                                           for k in ("vel", "dvort", "visc", "vort")],
        "p2d200k_vel_visc_w": [x["p2d_patch200k_winckelmans_vel"]["ginter_s"],
                               x["p2d_patch200k_winckelmans_visc"]["ginter_s"]],
        "f3d100k_vel_dvort": [x["f3d_sheet100k_vel"]["ginter_s"],
                              x["f3d_sheet100k_dvort_cube100k"]["ginter_s"]],
        "serving_light_p50_ms_served_plain": {r: [v["served"][0], v["plain"][0]]
                                              for r, v in light.items()},
        "serving_heavy_x": [v["x"] for v in heavy.values()],
        "cpu_baseline": out.get("cpu_baseline", {}).get("value")}


def headline_parity(p, vel, dv, args):
    """The timed step's last results on sampled targets: against the
    reference's CPU formulation (oracle, all sources) and against FP64."""
    import oracle
    idx = sample_idx(len(p))
    gv = vel.cpu().numpy()[idx]
    gd = dv.cpu().numpy()[idx]
    sub = p[idx].copy()
    rv = oracle.p3d_vel(p, sub["coord"], args.reg, SIGMA)
    rd = oracle.p3d_dvort(p, sub, args.reg, SIGMA)
    ev, ed = oracle.exact_p3d_vel_dvort(p, sub["coord"], sub["vorticity"], args.reg, SIGMA)
    return {"targets": len(idx), "vel_vs_reference": errs(gv, rv),
            "dvort_vs_reference": errs(gd, rd), "vel_vs_fp64": errs(gv, ev),
            "dvort_vs_fp64": errs(gd, ed), "reference_vs_fp64": {
                "vel": r4(errs(rv, ev)["rel_l2"]), "dvort": r4(errs(rd, ed)["rel_l2"])}}


def e2e_abi(cv, p, args):
    """Reference ABI with host buffers: cvtx_P3D_M2M_vel + cvtx_P3D_M2M_dvort."""
    from cvortex_gb300 import abi
    import oracle
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
    idx = sample_idx(n, seed=12)
    sub = p[idx].copy()
    ev, ed = oracle.exact_p3d_vel_dvort(p, sub["coord"], sub["vorticity"], args.reg, SIGMA)
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
            "fp64": {"vel": errs(o1[idx], ev), "dvort": errs(o2[idx], ed)},
            "fused_extension": {"value": r4(n * n / dtf / 1e9), "ms_per_step": r4(dtf * 1e3),
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


def rate(pairs, ms, flops, peak):
    return {"ginter_s": r4(pairs / ms / 1e6),
            "fp32_frac": r4(flops * pairs / (ms * 1e-3) / 1e12 / peak)}


def extras(cv, lib, args, torch, sh, peak):
    """Per-op rates on the scale-up, precision and batched workloads, each
    with its error against the FP64 oracle on sampled targets (rel L2 and
    max relative error per target)."""
    import oracle
    from cvortex_gb300 import workloads
    hbm_peak = measured_hbm_gbs()
    res = {}
    n = 100_000
    p = workloads.vortex_ring(n)
    idx = sample_idx(n)
    sub = p[idx].copy()
    rec = torch.from_numpy(p3d_records(p).reshape(n, 8)).cuda()
    o1 = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    o2 = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    for rname, r in REG.items():
        row = {}
        ev, ed = oracle.exact_p3d_vel_dvort(p, sub["coord"], sub["vorticity"], rname, SIGMA)
        for op, (a, b) in {"vel": (o1, None), "dvort": (None, o2), "veldvort": (o1, o2)}.items():
            f = lambda: lib.cvtx_gb300_dev_P3D_M2M(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                   a.data_ptr() if a is not None else None,
                                                   b.data_ptr() if b is not None else None,
                                                   r, SIGMA, sh)
            ms = timed_dev(f, torch, 5)
            row[op] = rate(n * n, ms, FLOPS[(op, r)], peak)
            e = []
            if a is not None:
                e.append(errs(a.cpu().numpy()[idx], ev)["rel_l2"])
            if b is not None:
                e.append(errs(b.cpu().numpy()[idx], ed)["rel_l2"])
            row[op]["fp64_rel_l2"] = max(e)
        if r in VISC_FLOPS:
            f = lambda: lib.cvtx_gb300_dev_P3D_M2M_visc(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                        o1.data_ptr(), r, SIGMA, 1e-3, sh)
            ms = timed_dev(f, torch, 5)
            row["visc"] = rate(n * n, ms, VISC_FLOPS[r], peak)
            row["visc"]["fp64_rel_l2"] = errs(o1.cpu().numpy()[idx],
                                              oracle.exact_p3d_visc(p, sub, rname, SIGMA, 1e-3))["rel_l2"]
        if r in VORT_FLOPS:
            f = lambda: lib.cvtx_gb300_dev_P3D_M2M_vort(rec.data_ptr(), n, rec.data_ptr(), 2, n,
                                                        o1.data_ptr(), r, SIGMA, sh)
            ms = timed_dev(f, torch, 5)
            row["vort"] = rate(n * n, ms, VORT_FLOPS[r], peak)
            row["vort"]["fp64_rel_l2"] = errs(o1.cpu().numpy()[idx],
                                              oracle.exact_p3d_vort(p, sub["coord"], rname, SIGMA))["rel_l2"]
        res[f"ring{n // 1000}k_{rname}"] = row
    del rec, o1, o2
    q = workloads.gaussian_patch_2d(200_000)
    nq = len(q)
    qi = sample_idx(nq)
    rq = torch.from_numpy(np.ascontiguousarray(
        np.stack([q["coord"][:, 0], q["coord"][:, 1], q["vorticity"], q["area"]], 1))).cuda()
    o = torch.empty((nq, 2), dtype=torch.float32, device="cuda")
    for rname, r, fl in (("gaussian", 3, 13), ("winckelmans", 1, 15)):
        f = lambda: lib.cvtx_gb300_dev_P2D_M2M_vel(rq.data_ptr(), nq, rq.data_ptr(), nq,
                                                   o.data_ptr(), r, SIGMA, sh)
        ms = timed_dev(f, torch, 5)
        res[f"p2d_patch200k_{rname}_vel"] = rate(nq * nq, ms, fl, peak)
        res[f"p2d_patch200k_{rname}_vel"]["fp64_rel_l2"] = errs(
            o.cpu().numpy()[qi], oracle.exact_p2d_vel(q, q["coord"][qi], rname, SIGMA))["rel_l2"]
    ov = torch.empty((nq,), dtype=torch.float32, device="cuda")
    for rname, r, fl in (("winckelmans", 1, 16), ("gaussian", 3, 10)):
        f = lambda: lib.cvtx_gb300_dev_P2D_M2M_visc(rq.data_ptr(), nq, rq.data_ptr(), nq,
                                                    ov.data_ptr(), r, SIGMA, 1e-3, sh)
        ms = timed_dev(f, torch, 5)
        res[f"p2d_patch200k_{rname}_visc"] = rate(nq * nq, ms, fl, peak)
        ex = oracle.exact_p2d_visc(q, q[qi], rname, SIGMA, 1e-3)
        res[f"p2d_patch200k_{rname}_visc"]["fp64_rel_l2"] = errs(ov.cpu().numpy()[qi], ex)["rel_l2"]
        # the reference's own FP32 pair formula carries most of this error
        res[f"p2d_patch200k_{rname}_visc"]["reference_fp64_rel_l2"] = errs(
            oracle.p2d_visc(q, q[qi], rname, SIGMA, 1e-3), ex)["rel_l2"]
    del rq, o, ov
    nf = 100_000
    fil = workloads.wake_sheet(nf)
    pts = workloads.sheet_targets(nf)
    fi = sample_idx(nf)
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
    res["f3d_sheet100k_vel"] = rate(nf * nf, ms, 51, peak)
    res["f3d_sheet100k_vel"]["fp64_rel_l2"] = errs(
        of.cpu().numpy()[fi], oracle.exact_f3d_vel(fil, pts[fi]))["rel_l2"]
    cube = workloads.uniform_cube(nf, seed=12)
    rc = torch.from_numpy(p3d_records(cube).reshape(nf, 8)).cuda()
    f = lambda: lib.cvtx_gb300_dev_F3D_M2M_dvort(rfd.data_ptr(), nf, rc.data_ptr(), 2, nf,
                                                 of.data_ptr(), sh)
    ms = timed_dev(f, torch, 3)
    res["f3d_sheet100k_dvort_cube100k"] = rate(nf * nf, ms, 62, peak)
    res["f3d_sheet100k_dvort_cube100k"]["fp64_rel_l2"] = errs(
        of.cpu().numpy()[fi], oracle.exact_f3d_dvort(fil, cube[fi]))["rel_l2"]
    # influence matrix: 25,000 points x 20,000 filaments, 4 B per entry
    nm, ni = INF_SHAPE
    dirs = np.zeros((nm, 4), np.float32)
    dirs[:, 2] = 1.0
    dd = torch.from_numpy(dirs).cuda()
    om = torch.empty((nm, ni), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_F3D_inf_mtrx(rfd.data_ptr(), ni, tfd.data_ptr(), dd.data_ptr(),
                                                nm, om.data_ptr(), sh)
    ms = timed_dev(f, torch, 5)
    gbs = 4.0 * nm * ni / (ms * 1e-3) / 1e9
    rows = sample_idx(nm, 64)
    res["f3d_inf_mtrx_25kx20k"] = {
        "ms": r4(ms), "write_gbs": r4(gbs), "hbm_frac": r4(gbs / hbm_peak) if hbm_peak else None,
        "fp32_frac": r4(INF_FLOPS * nm * ni / (ms * 1e-3) / 1e12 / peak),
        "fp64_rel_l2": errs(om.cpu().numpy()[rows], oracle.exact_f3d_vel(
            fil[:ni], pts[rows], dirs[rows, :3]))["rel_l2"]}
    del om, rfd, tfd, rc, of
    res["batch512"] = batch_extra(cv, lib, torch, sh)
    res["redistribute_ring200k_m4p"] = redistribute_extra(cv, lib)
    # the precision configuration's input: Gaussian, sigma 0.01, 1 % twins
    # closer than 1e-3 sigma; errors on sampled targets plus twins
    m = 1_000_000
    tw = workloads.cube_with_twins(m, 0.01)
    rb = torch.from_numpy(p3d_records(tw).reshape(m, 8)).cuda()
    b1 = torch.empty((m, 3), dtype=torch.float32, device="cuda")
    b2 = torch.empty((m, 3), dtype=torch.float32, device="cuda")
    f = lambda: lib.cvtx_gb300_dev_P3D_M2M(rb.data_ptr(), m, rb.data_ptr(), 2, m, b1.data_ptr(),
                                           b2.data_ptr(), 3, 0.01, sh)
    ms = timed_dev(f, torch, 2)
    ti = np.unique(np.concatenate([sample_idx(m, 192, seed=13), np.arange(m - 64, m)]))
    ev, ed = oracle.exact_p3d_vel_dvort(tw, tw["coord"][ti], tw["vorticity"][ti], "gaussian", 0.01)
    res["twins1M_gaussian_veldvort"] = rate(m * m, ms, FLOPS[("veldvort", 3)], peak)
    res["twins1M_gaussian_veldvort"].update(
        {"ms": r4(ms), "vel_fp64": errs(b1.cpu().numpy()[ti], ev),
         "dvort_fp64": errs(b2.cpu().numpy()[ti], ed), "targets_checked": int(len(ti))})
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
    gpu_out = out[:m_gpu].copy()
    cv.set_accelerated(False)
    try:
        m_host, t_host = run()
    finally:
        cv.set_accelerated(True)
    if m_gpu != m_host or gpu_out.tobytes() != out[:m_host].tobytes():
        raise RuntimeError("redistribution: GPU and host paths disagree")
    return {"particles_out": int(m_gpu), "gpu_ms": r4(t_gpu * 1e3), "host_ms": r4(t_host * 1e3),
            "host_cores": cpu_cores(), "speedup": r4(t_host / t_gpu),
            "gpu_equals_host": True}


def batch_extra(cv, lib, torch, sh, count=512):
    """512 independent vel+dvort problems (uniform cube each, Winckelmans,
    sigma 0.05), sizes log-uniform in [1,000, 50,000]: one plain device call
    per problem vs the batched persistent launch (autotuned, graph-captured).
    The batched results of the three largest and three random problems are
    checked against FP64 on sampled targets."""
    import oracle
    from cvortex_gb300 import abi, workloads
    sizes = workloads.batch_sizes(count)
    keep, probs, parts = [], [], []
    for i, n in enumerate(sizes):
        n = int(n)
        p = workloads.uniform_cube(n, seed=10_000 + i)
        rec = torch.from_numpy(p3d_records(p).reshape(n, 8)).cuda()
        v = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        d = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        keep.append((n, rec, v, d))
        parts.append(p)
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
    for _, _, v, d in keep:
        v.fill_(float("nan"))
        d.fill_(float("nan"))
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
    order = np.argsort(sizes)
    chk = list(order[-3:]) + list(np.random.Generator(np.random.PCG64(14)).choice(count, 3, False))
    worst = {"vel": 0.0, "dvort": 0.0}
    for i in chk:
        n, _, v, d = keep[i]
        ti = sample_idx(n, 64, seed=int(i))
        sub = parts[i][ti]
        ev, ed = oracle.exact_p3d_vel_dvort(parts[i], sub["coord"], sub["vorticity"],
                                            "winckelmans", SIGMA)
        worst["vel"] = max(worst["vel"], errs(v.cpu().numpy()[ti], ev)["rel_l2"])
        worst["dvort"] = max(worst["dvort"], errs(d.cpu().numpy()[ti], ed)["rel_l2"])
    return {"problems": count, "sizes": [int(sizes.min()), int(sizes.max())],
            "plain_ginter_s": r4(pairs / ms_plain / 1e6),
            "plain_separate_ginter_s": r4(pairs / ms_plain_sep / 1e6),
            "batched_ms": r4(ms_batch), "batched_ginter_s": r4(pairs / ms_batch / 1e6),
            "speedup": r4(ms_plain / ms_batch), "speedup_vs_separate": r4(ms_plain_sep / ms_batch),
            "tuned": [tpt.value, nt.value, chunk.value], "graph": bool(graph.value),
            "tune_s": r4(tune_s), "fp64_rel_l2_worst_of_6": {k: r4(x) for k, x in worst.items()}}


SERVE_RATES = (100, 300, 1000, 3000, 5000)
LIGHT_RATES = (100, 300, 1000)


def plain_measured(cv, kinds, inputs, arrival, steps, dt):
    """Plain per-request ABI calls served by one worker thread in arrival
    order: each request waits for its arrival time, then runs its `steps`
    steps through the reference ABI with host buffers (cvtx_P3D_M2M_vel +
    cvtx_P3D_M2M_dvort / cvtx_P2D_M2M_vel / cvtx_F3D_M2M_vel, Euler update
    on the host). Returns (latencies in ms, span in s)."""
    lat = []
    t0 = time.perf_counter()
    for t_arr, k, (a, b) in zip(arrival, kinds, inputs):
        now = time.perf_counter() - t0
        if now < t_arr:
            time.sleep(t_arr - now)
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
        lat.append((time.perf_counter() - t0 - t_arr) * 1e3)
    span = time.perf_counter() - t0 - arrival[0]
    if cv.last_error():
        raise RuntimeError(cv.last_error())
    return np.array(lat), span


def pct(x, q):
    return float(np.percentile(x, q, method="inverted_cdf"))


def serve_stream_run(cv, lib, count, lo, hi, rates, steps, dt):
    """One served stream (Poisson arrivals, 60/25/15 mix of P3D vel+dvort,
    P2D vel, F3D vel, sizes log-uniform on [lo, hi], `steps` resident
    forward-Euler steps per client) at each rate, and the same arrivals
    through plain per-request ABI calls (measured, one worker thread)."""
    from cvortex_gb300 import serve, workloads
    arrival, kinds, sizes, seeds = workloads.serve_stream(count, rate=1.0, lo=lo, hi=hi)
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
    res = {"requests": count, "sizes": [int(sizes.min()), int(sizes.max())],
           "mix": [int((kinds == i).sum()) for i in range(3)], "interactions": r4(pairs)}
    srv = serve.Server(lib, n_slots=32)
    served = {}
    try:
        warm = build()[:4]                        # first-use costs out of the timed runs
        for r in warm:
            srv.submit(r)
        srv.drain()
        for rt in rates:
            srv.reset_stats()
            srv.replay(build(), arrival / rt)
            if not srv.drain(600_000):
                raise RuntimeError("serving drain timed out")
            st = srv.stats()
            if st["completed"] != count:
                raise RuntimeError(f"served {st['completed']}/{count}: {cv.last_error()}")
            served[rt] = st
    finally:
        srv.close()
    res["rates"] = {}
    for rt in rates:
        st = served[rt]
        lat, span = plain_measured(cv, kinds, inputs, arrival / rt, steps, dt)
        s_g = st["interactions"] / st["span_s"] / 1e9
        p_g = pairs / span / 1e9
        res["rates"][str(rt)] = {
            "served": [r4(st["p50_ms"]), r4(st["p99_ms"]), r4(s_g)],
            "plain": [r4(pct(lat, 50)), r4(pct(lat, 99)), r4(p_g)],
            "x": r4(s_g / p_g)}
    return res


def serve_extra(cv, lib, count=64, steps=10, dt=1e-3):
    """Served mixed-size streams vs plain per-request ABI calls: the
    benchmark's stream (sizes 500-200,000, far above the GPU's capacity at
    every rate, so latency is queueing) and a light stream (sizes
    500-20,000) whose offered load stays below capacity at 100-300 req/s.
    Per rate: served and plain [p50 ms, p99 ms, G interactions/s], and x =
    served / plain interactions/s; plain latencies are measured."""
    out = {"fields": "[p50_ms, p99_ms, Ginteractions/s]",
           "light": serve_stream_run(cv, lib, count, 500, 20_000, LIGHT_RATES, steps, dt),
           "stream": serve_stream_run(cv, lib, count, 500, 200_000, SERVE_RATES, steps, dt)}
    out["served_one_p3d_fp64"] = served_one_check(lib)
    return out


def served_one_check(lib, n=200_000):
    """One served P3D request of 200,000 particles (one step), its velocity
    on sampled targets against FP64."""
    import oracle
    from cvortex_gb300 import serve, workloads
    p = workloads.uniform_cube(n, seed=31)
    with serve.Server(lib, n_slots=2) as srv:
        req = serve.Request.p3d(p, n_steps=1, dt=1e-3)
        rid = srv.submit(req)
        if not rid or srv.wait(rid, 120_000) != 0:
            raise RuntimeError("served check request failed")
    ti = sample_idx(n, 128, seed=15)
    ev, _ = oracle.exact_p3d_vel_dvort(p, p["coord"][ti], None, "winckelmans", SIGMA,
                                       want_dvort=False)
    return errs(req.vel_out[ti], ev)


# ---- reference arm ---------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_cores()))
    os.environ.setdefault("OMP_PROC_BIND", "spread")
    kind, ref = cpu_reference()
    p = workload(args)
    order = np.random.Generator(np.random.PCG64(7)).permutation(args.n)
    # size each step's target sample so that all K steps take about a minute
    probe = p[np.sort(order[:32])].copy()
    for _ in range(max(args.warmup, 1)):
        t0 = time.perf_counter()
        cpu_step(kind, ref, p, probe, args.reg)
        per_target = (time.perf_counter() - t0) / len(probe)
    budget_s = 60.0
    m = int(budget_s / max(args.steps, 1) / max(per_target, 1e-9))
    m = max(32, min(CPU_SAMPLE_TARGETS, m, args.n))
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
           "config": {"workload": workload_name(args),
                      "interactions_per_step": float(args.n) * args.n,
                      "sampled_interactions_per_step": float(len(sub)) * len(p),
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
