"""Continuous-batching request loop for surface spectra.

Models stay resident on the device; each in-flight batch runs on its own
engine (``Engine``: workspace, stream and staging of its own), so a batch is
admitted as soon as an engine is free, while other batches are still on the
GPU, and their kernels overlap on the device.  The number of engines is set
by free HBM at start-up (each engine's device bytes are known after the first
one is built).  A batch takes waiting requests first-come first-served up to
an engine's point capacity; each point's result depends only on its own
inputs (one persistent kernel solves every point independently), so a
request's result is the same alone and in any mix.

Nothing here computes the path: the engines run the CUDA kernels.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future

import numpy as np

from .api import ACCURACY_REF, ITERMAX_REF, PREC_FP64, Engine


class Request:
    """One surface-spectrum request: points (k, omega) of one model at one eta."""

    __slots__ = ("model", "kpts", "omega", "eta", "t_submit", "t_start", "t_done", "future")

    def __init__(self, model: int, kpts, omega, eta):
        self.model = int(model)
        self.omega = np.asarray(omega, np.float64).ravel()
        k = np.asarray(kpts, np.float64).reshape(-1, 2)
        if len(k) == 1 and len(self.omega) > 1:
            k = np.repeat(k, len(self.omega), axis=0)
        if len(k) != len(self.omega):
            raise ValueError("kpts and omega must give one k per point (or one k for all)")
        self.kpts = k
        self.eta = float(eta)
        self.t_submit = self.t_start = self.t_done = 0.0
        self.future: Future = Future()

    @property
    def npts(self) -> int:
        return len(self.omega)


class SurfaceServer:
    """Request loop over ``slots`` engines for a fixed set of resident models.

    ``engine_factory(max_points)`` builds one engine (by default an ``Engine``
    of ``models``); it is a parameter so that the scheduling can be tested
    without a GPU."""

    def __init__(self, models=None, tops=None, bots=None, precision: int = PREC_FP64,
                 slot_points: int = 1024, max_slots: int = 4, hbm_fraction: float = 0.5,
                 tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF, divide_by_pi: bool = False,
                 engine_factory=None, free_bytes=None):
        self.slot_points = int(slot_points)
        self.tol, self.itermax, self.divide_by_pi = tol, itermax, divide_by_pi
        if engine_factory is None:
            def engine_factory(n):
                return Engine(models, tops, bots, precision=precision, max_points=n)
        first = engine_factory(self.slot_points)
        per = max(1, int(first.info().get("device_bytes", 1)))
        if free_bytes is None:
            import torch
            free_bytes = torch.cuda.mem_get_info()[0] if torch.cuda.is_available() else per * max_slots
        n = int(max(1, min(max_slots, 1 + (hbm_fraction * free_bytes) // per)))
        self.engines = [first] + [engine_factory(self.slot_points) for _ in range(n - 1)]
        self._free = collections.deque(range(len(self.engines)))
        self._pending: collections.deque[Request] = collections.deque()
        self._cv = threading.Condition()
        self._stop = False
        self.batches: list[tuple[int, int]] = []      # (engine, points) per launched batch
        self._dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self._dispatcher.start()

    # -- client side -----------------------------------------------------------
    def submit(self, model: int, kpts, omega, eta) -> Future:
        r = Request(model, kpts, omega, eta)
        if r.npts > self.slot_points:
            raise ValueError(f"request of {r.npts} points exceeds the slot capacity {self.slot_points}")
        r.t_submit = time.perf_counter()
        with self._cv:
            if self._stop:
                raise RuntimeError("server closed")
            self._pending.append(r)
            self._cv.notify_all()
        return r.future

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        self._dispatcher.join()
        for e in self.engines:
            close = getattr(e, "close", None)
            if close:
                close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scheduling -----------------------------------------------------------
    def _take_batch(self) -> list[Request]:
        """Waiting requests, first come first served, up to one slot's points."""
        batch, n = [], 0
        while self._pending and n + self._pending[0].npts <= self.slot_points:
            r = self._pending.popleft()
            batch.append(r)
            n += r.npts
        return batch

    def _dispatch(self):
        workers = []
        while True:
            with self._cv:
                while not self._stop and not (self._pending and self._free):
                    self._cv.wait()
                if self._stop and not self._pending:
                    break
                if not self._free:
                    continue
                slot = self._free.popleft()
                batch = self._take_batch()
            t = threading.Thread(target=self._run, args=(slot, batch), daemon=True)
            t.start()
            workers.append(t)
            workers = [w for w in workers if w.is_alive()]
        for w in workers:
            w.join()

    def _run(self, slot: int, batch: list[Request]):
        t0 = time.perf_counter()
        try:
            pm = np.concatenate([np.full(r.npts, r.model, np.int32) for r in batch])
            k = np.concatenate([r.kpts for r in batch])
            om = np.concatenate([r.omega for r in batch])
            et = np.concatenate([np.full(r.npts, r.eta) for r in batch])
            for r in batch:
                r.t_start = t0
            out = self.engines[slot].run(pm, k, om, et, tol=self.tol, itermax=self.itermax,
                                         divide_by_pi=self.divide_by_pi)
            t1 = time.perf_counter()
            with self._cv:
                self.batches.append((slot, int(len(pm))))
            o = 0
            for r in batch:
                res = {name: v[o:o + r.npts].copy() for name, v in out.items()}
                o += r.npts
                r.t_done = t1
                res["latency_s"] = t1 - r.t_submit
                r.future.set_result(res)
        except BaseException as e:  # noqa: BLE001 - handed to the waiting clients
            for r in batch:
                if not r.future.done():
                    r.future.set_exception(e)
        finally:
            with self._cv:
                self._free.append(slot)
                self._cv.notify_all()


def poisson_requests(rng: np.random.Generator, nmodels: int, rate: float, n: int,
                     npts_range=(50, 400), omega_ev=(-1.0, 1.0), eta_ev=(1e-3, 1e-2)):
    """n requests with exponential inter-arrival times (mean 1/rate s): each a
    random model, one random in-plane k and an evenly spaced window of 50-400
    omegas inside omega_ev, eta log-uniform in eta_ev (energies in eV)."""
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    out = []
    for i in range(n):
        m = int(rng.integers(nmodels))
        npts = int(rng.integers(npts_range[0], npts_range[1] + 1))
        w0, w1 = np.sort(rng.uniform(omega_ev[0], omega_ev[1], 2))
        om = np.linspace(w0, w1, npts)
        k = rng.uniform(-0.5, 0.5, (1, 2))
        eta = float(np.exp(rng.uniform(np.log(eta_ev[0]), np.log(eta_ev[1]))))
        out.append((float(t[i]), m, k, om, eta))
    return out


def replay(server: SurfaceServer, reqs, ev2hartree: float) -> dict:
    """Submit requests at their arrival times; wait for all; throughput and
    latency percentiles."""
    t0 = time.perf_counter()
    futs = []
    for (ta, m, k, om, eta) in reqs:
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        futs.append(server.submit(m, k, om * ev2hartree, eta * ev2hartree))
    res = [f.result() for f in futs]
    wall = time.perf_counter() - t0
    lat = np.array([r["latency_s"] for r in res])
    pts = sum(len(r["dos_l"]) for r in res)
    return {"requests": len(res), "points": int(pts), "wall_s": wall, "solves_per_s": pts / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "flagged": int(sum(int((r["status"] != 0).sum()) for r in res)), "results": res}
