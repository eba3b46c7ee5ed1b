"""Serving loop on CPU: admission, rejection, simulated out-of-memory,
ordering and statistics of the scheduler, run without a GPU (dry-run mode:
admitted requests complete without computing). The GPU path of the same
scheduler is covered by test_gpu_serve.py."""
import threading

import numpy as np
import pytest

from cvortex_gb300 import serve, workloads


@pytest.fixture()
def dry(cv):
    with serve.Server(cv.lib, n_slots=4, hbm_bytes=1 << 20, dry_run=True) as s:
        yield s


def _p3d(n, seed=0, **kw):
    return serve.Request.p3d(workloads.uniform_cube(n, seed), **kw)


def test_invalid_requests_are_refused(dry):
    r = _p3d(10)
    r.reg = 7
    assert dry.submit(r) == 0
    r = _p3d(10, n_steps=0)
    assert dry.submit(r) == 0
    r = serve.Request(serve.F3D, np.zeros((4, 8), np.float32))     # no tracer points
    assert dry.submit(r) == 0
    assert dry.stats()["submitted"] == 0


def test_request_larger_than_budget_is_rejected(dry):
    big = _p3d(30_000)           # 30,000 x 56 B > 1 MiB budget
    small = _p3d(1000)
    ib, i_s = dry.submit(big), dry.submit(small)
    assert dry.wait(ib, 5000) == -1
    assert dry.wait(i_s, 5000) == 0
    st = dry.stats()
    assert st["rejected"] == 1 and st["completed"] == 1
    assert st["hbm_budget"] == 1 << 20
    assert st["interactions"] == pytest.approx(1000.0 * 1000 * 10)


def test_simulated_oom_rejects_when_nothing_can_free_memory(dry):
    dry.inject_alloc_failures(1)
    a, b = dry.submit(_p3d(100)), dry.submit(_p3d(100))
    assert dry.wait(a, 5000) == -2      # oom
    assert dry.wait(b, 5000) == 0
    st = dry.stats()
    assert st["rejected"] == 1 and st["completed"] == 1


def test_completion_statistics(dry):
    ids = [dry.submit(_p3d(200 + i)) for i in range(20)]
    assert dry.drain(10_000)
    for i in ids:
        st, lat, q = dry.info(i)
        assert st == 0 and lat >= 0 and 0 <= q <= lat
    s = dry.stats()
    assert s["completed"] == 20 and s["queued"] == 0 and s["in_flight"] == 0
    assert 0 <= s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert s["hbm_used"] == 0 and 0 < s["hbm_peak"] <= s["hbm_budget"]
    dry.reset_stats()
    assert dry.stats()["completed"] == 0
    assert dry.info(ids[0])[0] == -5      # forgotten


def test_concurrent_submitters(dry):
    ids, lock = [], threading.Lock()

    def worker(k):
        for i in range(25):
            kind = (k + i) % 3
            if kind == 0:
                r = _p3d(50 + i)
            elif kind == 1:
                r = serve.Request.p2d(workloads.gaussian_patch_2d(60 + i))
            else:
                r = serve.Request.f3d(workloads.wake_sheet(40 + i), workloads.sheet_targets(30))
            rid = dry.submit(r)
            with lock:
                ids.append(rid)

    th = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert dry.drain(10_000)
    assert len(set(ids)) == 100 and 0 not in ids
    assert all(dry.info(i)[0] == 0 for i in ids)
    assert dry.stats()["completed"] == 100


def test_replay_paces_arrivals(dry):
    reqs = [_p3d(100 + i) for i in range(5)]
    t = np.array([0.0, 0.01, 0.02, 0.03, 0.04])
    ids = dry.replay(reqs, t)
    assert dry.drain(10_000)
    s = dry.stats()
    assert s["completed"] == 5 and s["span_s"] >= 0.035
    assert sorted(ids) == ids


def test_served_stream_mix():
    arr, kinds, sizes, seeds = workloads.serve_stream(4000, rate=1000.0)
    assert np.all(np.diff(arr) >= 0) and arr[0] == 0.0
    frac = np.bincount(kinds, minlength=3) / len(kinds)
    assert np.allclose(frac, workloads.SERVE_MIX, atol=0.03)
    assert sizes.min() >= 500 and sizes.max() <= 200_000
    assert abs(np.mean(np.diff(arr)) - 1e-3) < 1e-4
