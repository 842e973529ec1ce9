"""Request-loop scheduling without a GPU: a fake engine stands in for the
CUDA engine (its run() returns values computed from each point's own inputs
and sleeps to look busy), and fake models carry only an Ndim, so these tests
cover admission by the device-memory budget, engine tiers, continuous
batching, models added while serving, and result routing."""
import threading
import time

import numpy as np
import pytest

from wannier_tools_gb300.serving import SurfaceServer, poisson_requests, replay


class FakeModel:
    def __init__(self, ndim):
        self.ndim = ndim
        self.nw = ndim


class FakeEngine:
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, models, max_points, busy_s=0.02, nbytes=1000):
        self.models = list(models)
        self.max_points = max_points
        self.busy_s = busy_s
        self.nbytes = nbytes
        self.closed = False
        self.runs = 0

    def info(self):
        return {"device_bytes": self.nbytes, "max_points": self.max_points, "launches": self.runs}

    def run(self, pm, k, om, et, tol, itermax, divide_by_pi):
        assert len(pm) <= self.max_points and not self.closed
        assert pm.min() >= 0 and pm.max() < len(self.models)      # engine-local model indices
        with FakeEngine.lock:
            FakeEngine.live += 1
            FakeEngine.peak = max(FakeEngine.peak, FakeEngine.live)
        time.sleep(self.busy_s)
        with FakeEngine.lock:
            FakeEngine.live -= 1
        self.runs += 1
        n = len(pm)
        # the value depends on the model's Ndim (not on its engine-local index)
        nd = np.array([self.models[i].ndim for i in pm], float)
        return {"dos_l": nd + k[:, 0] + om, "dos_r": k[:, 1] * et, "dos_bulk": om * 2.0,
                "iters": np.full(n, 7, np.int32), "status": np.zeros(n, np.uint8)}

    def close(self):
        self.closed = True


def tier_bytes(tier, n):
    return tier * 10            # tier 64: 640 bytes, tier 320: 3200 bytes


def make_server(models, budget, busy=None, **kw):
    busy = busy or {}

    def factory(ms, ts, bs, n):
        tier = max(m.ndim for m in ms)
        return FakeEngine(ms, n, busy_s=busy.get(max(m.ndim for m in ms), 0.02),
                          nbytes=tier_bytes(next(t for t in (64, 128, 192, 320) if tier <= t), n))
    return SurfaceServer(models, engine_factory=factory, bytes_estimate=tier_bytes,
                         budget_bytes=budget, **kw)


def expected(ndim, k, om, eta):
    k = np.repeat(np.asarray(k).reshape(-1, 2), len(om), axis=0)
    return ndim + k[:, 0] + om, k[:, 1] * eta, om * 2.0


def test_results_routed_and_batches_bounded():
    rng = np.random.default_rng(0)
    FakeEngine.peak = 0
    models = [FakeModel(16), FakeModel(40), FakeModel(112)]
    srv = make_server(models, budget=10 ** 6, slot_points=100, max_slots=3)
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
            dl, dr, db = expected(models[m].ndim, k, om, eta)
            assert np.allclose(r["dos_l"], dl) and np.allclose(r["dos_r"], dr)
            assert np.allclose(r["dos_bulk"], db) and r["latency_s"] >= 0
        assert all(n <= 100 for _, n in srv.batches)
        assert sum(n for _, n in srv.batches) == sum(len(x[2]) for x in reqs)
        assert FakeEngine.peak >= 2          # batches overlapped on separate engines
        assert srv.engines_built <= 3
    finally:
        srv.close()


def test_engines_fit_the_budget_and_idle_ones_retire():
    """Budget for two small engines only: never more device bytes than the budget;
    a model added later, of a larger tier, retires the idle small engines to make
    room for its own."""
    small, mid = FakeModel(40), FakeModel(100)         # tiers 64 (640 B) and 128 (1280 B)
    srv = make_server([small], budget=1300, slot_points=64, max_slots=4)
    peak = [0]
    stop = threading.Event()

    def watch():
        while not stop.is_set():
            peak[0] = max(peak[0], srv.used_bytes())
            time.sleep(0.001)
    th = threading.Thread(target=watch)
    th.start()
    try:
        fs = [srv.submit(0, [[0.1, 0.2]], np.linspace(0, 1, 30), 1e-3) for _ in range(6)]
        for f in fs:
            f.result(timeout=30)
        assert srv.engines_built == 2                   # two tier-64 engines fit 1300 bytes
        assert srv.add_model(mid) == 1
        g = srv.submit(1, [[0.1, 0.2]], np.linspace(0, 1, 30), 1e-3)   # needs 1280 bytes
        g.result(timeout=30)
        assert srv.engines_retired >= 2                 # both idle small engines made room
    finally:
        stop.set()
        th.join()
        srv.close()
    assert peak[0] <= 1300


def test_large_request_waits_while_small_ones_proceed():
    """Budget 3200: three busy tier-64 engines (1920 B) leave no room for the
    tier-320 engine (3200 B) of a large model added while they run.  The large
    request waits; small requests that arrive after it run on the small engines
    as they free up; once its bypass time is over the small ones are held back,
    the small engines drain and retire, and the large request runs."""
    small, large = FakeModel(40), FakeModel(300)
    srv = make_server([small], budget=3200, busy={40: 0.15, 300: 0.05},
                      slot_points=64, max_slots=4, max_bypass_s=0.4)
    try:
        first = [srv.submit(0, [[0.1, 0.2]], np.linspace(0, 1, 60), 1e-3) for _ in range(3)]
        time.sleep(0.05)
        assert srv.add_model(large) == 1
        big = srv.submit(1, [[0.3, 0.1]], np.linspace(0, 1, 40), 1e-3)
        time.sleep(0.02)
        later = [srv.submit(0, [[0.2, 0.2]], np.linspace(0, 1, 60), 1e-3) for _ in range(2)]
        t_later = [f.result(timeout=30)["latency_s"] for f in later]
        rb = big.result(timeout=30)
        for f in first:
            f.result(timeout=30)
        # the small requests that came after the large one finished before it
        t_big_done = rb["latency_s"] + 0.0
        assert max(t_later) < t_big_done
        dl, _, _ = expected(300, [[0.3, 0.1]], np.linspace(0, 1, 40), 1e-3)
        assert np.allclose(rb["dos_l"], dl)
        assert srv.engines_retired >= 1
    finally:
        srv.close()


def test_old_blocked_request_holds_later_ones_back():
    """A stream of small requests cannot starve a large one: after max_bypass_s
    nothing younger starts until the large request has its engine."""
    small, large = FakeModel(40), FakeModel(300)
    srv = make_server([small], budget=3200, busy={40: 0.05, 300: 0.01},
                      slot_points=64, max_slots=4, max_bypass_s=0.2)
    try:
        stream = [srv.submit(0, [[0.1, 0.2]], np.linspace(0, 1, 60), 1e-3) for _ in range(3)]
        time.sleep(0.01)
        srv.add_model(large)
        big = srv.submit(1, [[0.3, 0.1]], np.linspace(0, 1, 40), 1e-3)
        t0 = time.perf_counter()
        while not big.done() and time.perf_counter() - t0 < 10:
            stream.append(srv.submit(0, [[0.1, 0.2]], np.linspace(0, 1, 60), 1e-3))
            time.sleep(0.01)
        assert big.done(), "the large request was starved"
        big.result(timeout=1)
        for f in stream:
            f.result(timeout=30)
    finally:
        srv.close()


def test_model_added_while_serving():
    m0 = FakeModel(16)
    srv = make_server([m0], budget=10 ** 6, slot_points=64, max_slots=3)
    try:
        a = srv.submit(0, [[0.1, 0.2]], np.linspace(0, 1, 20), 1e-3)
        a.result(timeout=30)
        built = srv.engines_built
        mid = srv.add_model(FakeModel(150))
        assert mid == 1
        b = srv.submit(mid, [[0.1, 0.2]], np.linspace(0, 1, 20), 1e-3)
        c = srv.submit(0, [[0.4, 0.2]], np.linspace(0, 1, 20), 1e-3)
        rb = b.result(timeout=30)
        dl, _, _ = expected(150, [[0.1, 0.2]], np.linspace(0, 1, 20), 1e-3)
        assert np.allclose(rb["dos_l"], dl)
        c.result(timeout=30)
        assert srv.engines_built > built                # an engine holding the new model
        with pytest.raises(ValueError):
            srv.submit(7, [[0.1, 0.2]], np.zeros(3), 1e-3)
    finally:
        srv.close()


def test_oversized_requests_rejected():
    srv = make_server([FakeModel(16), FakeModel(300)], budget=2000, slot_points=10, max_slots=1)
    try:
        with pytest.raises(ValueError):
            srv.submit(0, [[0.1, 0.2]], np.zeros(11), 1e-3)       # more points than a slot holds
        with pytest.raises(ValueError):
            srv.submit(1, [[0.1, 0.2]], np.zeros(5), 1e-3)        # its engine never fits 2000 B
        with pytest.raises(ValueError):
            srv.add_model(FakeModel(400))                          # above the largest tier
    finally:
        srv.close()


def test_engine_failure_reaches_clients():
    class Broken(FakeEngine):
        def run(self, *a, **k):
            raise RuntimeError("engine failed")
    srv = SurfaceServer([FakeModel(16)], engine_factory=lambda ms, ts, bs, n: Broken(ms, n),
                        bytes_estimate=tier_bytes, budget_bytes=10 ** 6, slot_points=10, max_slots=1)
    try:
        f = srv.submit(0, [[0.1, 0.2]], np.zeros(3), 1e-3)
        with pytest.raises(RuntimeError):
            f.result(timeout=10)
        # the engine is free again: a later request still runs (and fails the same way)
        with pytest.raises(RuntimeError):
            srv.submit(0, [[0.1, 0.2]], np.zeros(2), 1e-3).result(timeout=10)
    finally:
        srv.close()


def test_engine_build_failure_reaches_clients():
    def factory(ms, ts, bs, n):
        raise MemoryError("no device memory")
    srv = SurfaceServer([FakeModel(16)], engine_factory=factory, bytes_estimate=tier_bytes,
                        budget_bytes=10 ** 6, slot_points=10, max_slots=1)
    try:
        with pytest.raises(MemoryError):
            srv.submit(0, [[0.1, 0.2]], np.zeros(3), 1e-3).result(timeout=10)
        assert srv.used_bytes() == 0
    finally:
        srv.close()


def test_poisson_replay_reports_percentiles():
    rng = np.random.default_rng(3)
    reqs = poisson_requests(rng, nmodels=2, rate=400.0, n=30, npts_range=(5, 20))
    srv = make_server([FakeModel(8), FakeModel(30)], budget=10 ** 6, slot_points=64, max_slots=2)
    try:
        rep = replay(srv, reqs, ev2hartree=1.0)
    finally:
        srv.close()
    assert rep["requests"] == 30 and rep["points"] == sum(len(r[3]) for r in reqs)
    assert 0 <= rep["p50_ms"] <= rep["p99_ms"]
