"""Host-side front end of the serving loop (cvtx_gb300_server_* in
include/cvortex/cvtx_gb300.h): request construction from the reference's
record arrays, submission, waiting and statistics.

The reference has no serving API; its callers issue one blocking
cvtx_*_M2M call per request (src/P3D.cpp:343-366, src/P2D.cpp:115-140,
src/F3D.cpp:143-166). A served request carries its own state and runs
`n_steps` device-resident time steps (M2M, then forward Euler).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .abi import cvtx_gb300_request, cvtx_gb300_server_stats

P3D, P2D, F3D = 0, 1, 2
REG_IDS = {"singular": 0, "winckelmans": 1, "planetary": 2, "gaussian": 3}
STATUS = {0: "done", 1: "pending", 2: "running", -1: "rejected", -2: "oom", -3: "failed",
          -4: "timeout", -5: "unknown"}
DRY_RUN = 1


def p3d_records(p: np.ndarray) -> np.ndarray:
    """cvtx_P3D structured array -> (n, 8) records (x, y, z, vol, ax, ay, az, 0)."""
    r = np.zeros((len(p), 8), np.float32)
    r[:, 0:3] = p["coord"]
    r[:, 3] = p["volume"]
    r[:, 4:7] = p["vorticity"]
    return r


def p2d_records(p: np.ndarray) -> np.ndarray:
    """cvtx_P2D structured array -> (n, 4) records (x, y, Gamma, area)."""
    r = np.zeros((len(p), 4), np.float32)
    r[:, 0:2] = p["coord"]
    r[:, 2] = p["vorticity"]
    r[:, 3] = p["area"]
    return r


def f3d_records(f: np.ndarray) -> np.ndarray:
    """cvtx_F3D structured array -> (n, 8) records (start, strength, end, 0)."""
    r = np.zeros((len(f), 8), np.float32)
    r[:, 0:3] = f["start"]
    r[:, 3] = f["strength"]
    r[:, 4:7] = f["end"]
    return r


def point_records(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, np.float32)
    r = np.zeros((len(x), 4), np.float32)
    r[:, : x.shape[1]] = x
    return r


@dataclass
class Request:
    """One request and the host buffers it reads and writes (kept alive here)."""
    kind: int
    state_in: np.ndarray
    n_steps: int = 10
    dt: float = 1e-3
    reg: int = 1
    sigma: float = 0.05
    tgt_in: np.ndarray | None = None
    want_vel: bool = True
    state_out: np.ndarray = field(init=False)
    vel_out: np.ndarray | None = field(init=False)

    def __post_init__(self):
        self.state_in = np.ascontiguousarray(self.state_in, np.float32)
        if self.tgt_in is not None:
            self.tgt_in = np.ascontiguousarray(self.tgt_in, np.float32)
        out_src = self.tgt_in if self.kind == F3D else self.state_in
        if out_src is None:                     # F3D without tracer points (invalid)
            out_src = np.zeros((0, 4), np.float32)
        self.state_out = np.empty_like(out_src)
        width = 2 if self.kind == P2D else 3
        self.vel_out = np.empty((len(out_src), width), np.float32) if self.want_vel else None

    @classmethod
    def p3d(cls, particles, **kw):
        return cls(P3D, p3d_records(particles), **kw)

    @classmethod
    def p2d(cls, particles, **kw):
        return cls(P2D, p2d_records(particles), **kw)

    @classmethod
    def f3d(cls, filaments, points, **kw):
        return cls(F3D, f3d_records(filaments), tgt_in=point_records(points), **kw)

    @property
    def interactions(self) -> float:
        tg = len(self.tgt_in) if self.kind == F3D else len(self.state_in)
        return float(len(self.state_in)) * tg * self.n_steps

    def c_struct(self) -> cvtx_gb300_request:
        r = cvtx_gb300_request()
        r.kind, r.reg, r.sigma, r.dt = self.kind, self.reg, self.sigma, self.dt
        r.n_steps, r.n = self.n_steps, len(self.state_in)
        r.n_tgt = len(self.tgt_in) if self.tgt_in is not None else 0
        r.state_in = self.state_in.ctypes.data
        r.tgt_in = self.tgt_in.ctypes.data if self.tgt_in is not None else None
        r.state_out = self.state_out.ctypes.data
        r.vel_out = self.vel_out.ctypes.data if self.vel_out is not None else None
        return r


class Server:
    """Owns one cvtx_gb300_server."""

    def __init__(self, lib: C.CDLL, n_slots: int = 0, hbm_bytes: int = 0,
                 dry_run: bool = False):
        self.lib = lib
        self.h = lib.cvtx_gb300_server_create(n_slots, hbm_bytes, DRY_RUN if dry_run else 0)
        if not self.h:
            raise RuntimeError("cvtx_gb300_server_create failed: "
                               + (lib.cvtx_gb300_last_error() or b"").decode())
        self._live: dict[int, Request] = {}

    def submit(self, req: Request) -> int:
        cs = req.c_struct()
        rid = self.lib.cvtx_gb300_server_submit(self.h, C.byref(cs))
        if rid:
            self._live[rid] = req
        return rid

    def replay(self, reqs: list[Request], arrival_s) -> list[int]:
        """Submit reqs[i] at arrival_s[i] seconds from now (from C++, so the
        pacing does not depend on the interpreter)."""
        n = len(reqs)
        arr = (cvtx_gb300_request * n)(*[r.c_struct() for r in reqs])
        times = (C.c_double * n)(*[float(t) for t in arrival_s])
        ids = (C.c_ulonglong * n)()
        if self.lib.cvtx_gb300_server_replay(self.h, arr, times, n, ids) != 0:
            raise RuntimeError("cvtx_gb300_server_replay failed")
        out = list(ids)
        for rid, req in zip(out, reqs):
            if rid:
                self._live[rid] = req
        return out

    def wait(self, rid: int, timeout_ms: float = -1.0) -> int:
        return self.lib.cvtx_gb300_server_wait(self.h, rid, timeout_ms)

    def drain(self, timeout_ms: float = -1.0) -> bool:
        return self.lib.cvtx_gb300_server_drain(self.h, timeout_ms) == 0

    def info(self, rid: int):
        lat, q = C.c_double(), C.c_double()
        st = self.lib.cvtx_gb300_server_request_info(self.h, rid, C.byref(lat), C.byref(q))
        return st, lat.value, q.value

    def stats(self) -> dict:
        s = cvtx_gb300_server_stats()
        self.lib.cvtx_gb300_server_stats_get(self.h, C.byref(s))
        return s.as_dict()

    def reset_stats(self):
        self.lib.cvtx_gb300_server_reset_stats(self.h)
        self._live.clear()

    def inject_alloc_failures(self, count: int):
        self.lib.cvtx_gb300_server_inject_alloc_failures(self.h, count)

    def close(self):
        if self.h:
            self.lib.cvtx_gb300_server_destroy(self.h)
            self.h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
