"""Request-loop scheduling without a GPU: a fake engine stands in for the
CUDA engine (its run() returns values computed from each point's own inputs
and sleeps to look busy), so these tests cover admission, slot limits,
continuous batching and result routing."""
import threading
import time

import numpy as np
import pytest

from wannier_tools_gb300.serving import SurfaceServer, poisson_requests, replay


class FakeEngine:
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, max_points, busy_s=0.02):
        self.max_points = max_points
        self.busy_s = busy_s
        self.closed = False

    def info(self):
        return {"device_bytes": 1000, "max_points": self.max_points, "launches": 0}

    def run(self, pm, k, om, et, tol, itermax, divide_by_pi):
        assert len(pm) <= self.max_points
        with FakeEngine.lock:
            FakeEngine.live += 1
            FakeEngine.peak = max(FakeEngine.peak, FakeEngine.live)
        time.sleep(self.busy_s)
        with FakeEngine.lock:
            FakeEngine.live -= 1
        n = len(pm)
        return {"dos_l": pm + k[:, 0] + om, "dos_r": k[:, 1] * et, "dos_bulk": om * 2.0,
                "iters": np.full(n, 7, np.int32), "status": np.zeros(n, np.uint8)}

    def close(self):
        self.closed = True


def expected(m, k, om, eta):
    k = np.repeat(np.asarray(k).reshape(-1, 2), len(om), axis=0) if np.asarray(k).size == 2 else k
    return m + k[:, 0] + om, k[:, 1] * eta, om * 2.0


def test_slots_limited_by_free_memory():
    srv = SurfaceServer(engine_factory=lambda n: FakeEngine(n), slot_points=64, max_slots=8,
                        hbm_fraction=0.5, free_bytes=4500)
    try:
        assert len(srv.engines) == 1 + int(0.5 * 4500) // 1000     # 3
    finally:
        srv.close()
    assert all(e.closed for e in srv.engines)


def test_results_routed_and_batches_bounded():
    rng = np.random.default_rng(0)
    FakeEngine.peak = 0
    srv = SurfaceServer(engine_factory=lambda n: FakeEngine(n), slot_points=100, max_slots=3,
                        free_bytes=10 ** 6)
    reqs = []
    try:
        for i in range(40):
            n = int(rng.integers(5, 60))
            k = rng.uniform(-0.5, 0.5, (1, 2))
            om = rng.uniform(-1, 1, n)
            eta = float(rng.uniform(1e-3, 1e-2))
            reqs.append((i % 3, k, om, eta, srv.submit(i % 3, k, om, eta)))
        for m, k, om, eta, f in reqs:
            r = f.result(timeout=30)
            dl, dr, db = expected(m, k, om, eta)
            assert np.allclose(r["dos_l"], dl) and np.allclose(r["dos_r"], dr)
            assert np.allclose(r["dos_bulk"], db) and r["latency_s"] >= 0
        assert all(n <= 100 for _, n in srv.batches)
        assert sum(n for _, n in srv.batches) == sum(len(x[2]) for x in reqs)
        assert FakeEngine.peak >= 2          # batches overlapped on separate slots
    finally:
        srv.close()


def test_oversized_request_rejected():
    srv = SurfaceServer(engine_factory=lambda n: FakeEngine(n), slot_points=10, max_slots=1,
                        free_bytes=10 ** 6)
    try:
        with pytest.raises(ValueError):
            srv.submit(0, [[0.1, 0.2]], np.zeros(11), 1e-3)
    finally:
        srv.close()


def test_engine_failure_reaches_clients():
    class Broken(FakeEngine):
        def run(self, *a, **k):
            raise RuntimeError("engine failed")
    srv = SurfaceServer(engine_factory=lambda n: Broken(n), slot_points=10, max_slots=1,
                        free_bytes=10 ** 6)
    try:
        f = srv.submit(0, [[0.1, 0.2]], np.zeros(3), 1e-3)
        with pytest.raises(RuntimeError):
            f.result(timeout=10)
        # the slot is returned: a later request still runs (and fails the same way)
        with pytest.raises(RuntimeError):
            srv.submit(0, [[0.1, 0.2]], np.zeros(2), 1e-3).result(timeout=10)
    finally:
        srv.close()


def test_poisson_replay_reports_percentiles():
    rng = np.random.default_rng(3)
    reqs = poisson_requests(rng, nmodels=2, rate=400.0, n=30, npts_range=(5, 20))
    srv = SurfaceServer(engine_factory=lambda n: FakeEngine(n, busy_s=0.005), slot_points=64,
                        max_slots=2, free_bytes=10 ** 6)
    try:
        rep = replay(srv, reqs, ev2hartree=1.0)
    finally:
        srv.close()
    assert rep["requests"] == 30 and rep["points"] == sum(len(r[3]) for r in reqs)
    assert 0 <= rep["p50_ms"] <= rep["p99_ms"]
