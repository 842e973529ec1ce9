"""Continuous-batching request loop for surface spectra.

Models are registered with the server (at construction, or with ``add_model``
while it serves) and stay resident on the device.  Requests are admitted as
device memory and engines free up:

* An engine (``Engine``: the device tables of a model set, a workspace sized
  for the set's largest Ndim, its own stream and staging) serves one Ndim
  tier: the registered models whose Ndim is at most the tier's bound.  A
  request runs on an engine whose tier covers its model's Ndim and whose model
  set contains its model.  A new engine takes the largest tier (up to the
  largest registered model's) that fits the budget as it stands, so while
  memory allows every engine serves every model; a smaller tier is built,
  retiring idle engines, only when nothing larger fits.
* The server holds a device-memory budget (a fraction of the free HBM at
  start, or given).  An engine is built only when its device bytes fit what
  the existing engines leave of the budget; idle engines are retired (least
  recently used first) to make room, and at most ``max_slots`` engines exist.
  So a request of a large model waits while its engine does not fit, and
  requests of smaller models that fit keep running.  A request that has
  waited longer than ``max_bypass_s`` for memory holds every later request
  back until it is admitted (the running batches drain and free their
  engines), so it cannot be starved.
* Waiting requests are batched first come first served up to an engine's
  point capacity; batches run concurrently on different engines and their
  kernels overlap on the device.
* ``add_model`` registers a model while the server runs: engines built after
  it include the model; engines built before keep serving the models they
  hold.

Each point's result depends only on its own inputs (one persistent kernel
solves every point independently, with the same arithmetic in every engine),
so a request's result is the same alone and in any mix, on any engine.

Nothing here computes the path: the engines run the CUDA kernels.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future

import numpy as np

from .api import ACCURACY_REF, ITERMAX_REF, PREC_FP64, PREC_MIXED, Engine

DEFAULT_TIERS = (64, 128, 192, 320)


class Request:
    """One surface-spectrum request: points (k, omega) of one model at one eta."""

    __slots__ = ("model", "kpts", "omega", "eta", "t_submit", "t_start", "t_done", "future",
                 "t_blocked")

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
        self.t_blocked = None           # first time it could not be admitted for memory
        self.future: Future = Future()

    @property
    def npts(self) -> int:
        return len(self.omega)


class _Slot:
    """An engine of one tier over a fixed model set (global ids; local index = position)."""

    def __init__(self, tier: int, ids, nbytes: int):
        self.tier = tier
        self.ids = tuple(ids)
        self.local = {g: i for i, g in enumerate(self.ids)}
        self.bytes = int(nbytes)
        self.engine = None
        self.busy = True                 # a new slot is built and run by its first batch
        self.last_used = time.perf_counter()


def engine_bytes_estimate(tier: int, max_points: int, precision: int, nsm: int = 152) -> int:
    """Device bytes an engine of this tier holds: one workspace of 9 (FP64) or 11
    (mixed) tier x tier complex matrices per SM, plus its staging."""
    mats = 11 if precision == PREC_MIXED else 9
    return nsm * mats * tier * tier * 16 + max_points * 72 + (1 << 20)


class SurfaceServer:
    """Request loop over engines built on demand within a device-memory budget.

    ``engine_factory(models, tops, bots, max_points)`` builds one engine (by
    default an ``Engine``) and ``bytes_estimate(tier, max_points)`` gives the
    device bytes of an engine of that tier before it is built; both are
    parameters so that the scheduling can be tested without a GPU (models are
    then any objects with an ``ndim``)."""

    def __init__(self, models=None, tops=None, bots=None, precision: int = PREC_FP64,
                 slot_points: int = 1024, max_slots: int = 4, hbm_fraction: float = 0.5,
                 tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF, divide_by_pi: bool = False,
                 engine_factory=None, free_bytes=None, budget_bytes=None, tiers=DEFAULT_TIERS,
                 bytes_estimate=None, max_bypass_s: float = 2.0):
        self.slot_points = int(slot_points)
        self.max_slots = int(max_slots)
        self.precision = precision
        self.tol, self.itermax, self.divide_by_pi = tol, itermax, divide_by_pi
        self.tiers = tuple(sorted(tiers))
        self.max_bypass_s = float(max_bypass_s)
        if engine_factory is None:
            def engine_factory(ms, ts, bs, n):
                return Engine(ms, ts, bs, precision=precision, max_points=n)
        self._factory = engine_factory
        if bytes_estimate is None:
            nsm = 152
            try:
                import torch
                if torch.cuda.is_available():
                    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            except Exception:
                pass

            def bytes_estimate(tier, n):
                return engine_bytes_estimate(tier, n, precision, nsm)
        self._estimate = bytes_estimate
        if budget_bytes is None:
            if free_bytes is None:
                import torch
                free_bytes = torch.cuda.mem_get_info()[0] if torch.cuda.is_available() else 0
            budget_bytes = int(hbm_fraction * free_bytes)
        self.budget = int(budget_bytes)
        self._models = []                # (model, top, bot, ndim)
        self._slots: list[_Slot] = []
        self._pending: collections.deque[Request] = collections.deque()
        self._cv = threading.Condition()
        self._stop = False
        self._retired_launches = 0
        self.batches: list[tuple[int, int]] = []      # (tier, points) per launched batch
        self.engines_built = 0
        self.engines_retired = 0
        for i, m in enumerate(models or []):
            self.add_model(m, tops[i] if tops is not None else None, bots[i] if bots is not None else None)
        self._dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self._dispatcher.start()

    # -- models ---------------------------------------------------------------
    def add_model(self, model, top=None, bot=None) -> int:
        """Register a model (its TopOrbitals / BottomOrbitals lists, 1-based; all
        orbitals by default); returns its id for ``submit``.  Allowed while serving."""
        n = int(model.ndim)
        if n > self.tiers[-1]:
            raise ValueError(f"Ndim {n} above the largest tier {self.tiers[-1]}")
        nw = getattr(model, "nw", n)
        top = list(top) if top is not None else list(range(1, nw + 1))
        bot = list(bot) if bot is not None else list(range(1, nw + 1))
        with self._cv:
            self._models.append((model, top, bot, n))
            self._cv.notify_all()
            return len(self._models) - 1

    def tier_of(self, ndim: int) -> int:
        return next(t for t in self.tiers if ndim <= t)

    # -- client side -----------------------------------------------------------
    def submit(self, model: int, kpts, omega, eta) -> Future:
        r = Request(model, kpts, omega, eta)
        if r.npts > self.slot_points:
            raise ValueError(f"request of {r.npts} points exceeds the slot capacity {self.slot_points}")
        r.t_submit = time.perf_counter()
        with self._cv:
            if self._stop:
                raise RuntimeError("server closed")
            if not 0 <= r.model < len(self._models):
                raise ValueError(f"unknown model id {r.model}")
            need = int(self._estimate(self.tier_of(self._models[r.model][3]), self.slot_points))
            if need > self.budget:
                raise ValueError(f"an engine for model {r.model} needs {need} device bytes, more "
                                 f"than the server's budget of {self.budget}")
            self._pending.append(r)
            self._cv.notify_all()
        return r.future

    @property
    def engines(self):
        """The engines that exist now."""
        with self._cv:
            return [s.engine for s in self._slots if s.engine is not None]

    def launches(self) -> int:
        """Kernel launches of every engine this server has run, retired ones included."""
        with self._cv:
            live = [s.engine for s in self._slots if s.engine is not None]
            done = self._retired_launches
        return done + sum(int(e.info().get("launches", 0)) for e in live)

    def used_bytes(self) -> int:
        with self._cv:
            return sum(s.bytes for s in self._slots)

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        self._dispatcher.join()
        with self._cv:
            slots, self._slots = self._slots, []
        for s in slots:
            self._close_engine(s)
        self._closed_slots = slots

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scheduling (called with the lock held) ----------------------------------
    def _compatible(self, s: _Slot, r: Request) -> bool:
        return r.model in s.local and self._models[r.model][3] <= s.tier

    def _take_batch(self, s: _Slot, first: Request) -> list[Request]:
        """first, then later waiting requests the engine can run, first come first
        served, up to one slot's points."""
        batch, n = [first], first.npts
        self._pending.remove(first)
        for r in list(self._pending):
            if n + r.npts > self.slot_points:
                break
            if self._compatible(s, r):
                self._pending.remove(r)
                batch.append(r)
                n += r.npts
        return batch

    def _make_room(self, need: int) -> bool:
        """Retire idle engines, least recently used first, until `need` bytes and
        one more engine fit; False (nothing retired) if that is impossible."""
        idle = sorted((s for s in self._slots if not s.busy), key=lambda s: s.last_used)
        used = sum(s.bytes for s in self._slots)
        count = len(self._slots)
        drop = []
        for s in idle:
            if used + need <= self.budget and count < self.max_slots:
                break
            drop.append(s)
            used -= s.bytes
            count -= 1
        if used + need > self.budget or count >= self.max_slots:
            return False
        for s in drop:
            self._slots.remove(s)
            self._retire(s)
        return True

    def _plan(self):
        """(slot, batch, build) for the next batch, or None if nothing can start.
        Requests are tried in arrival order: on a free engine that can run them,
        else on a new engine if it fits the budget (retiring idle ones); a request
        that fits neither waits, and once it has waited longer than max_bypass_s
        no later request starts before it."""
        now = time.perf_counter()
        for r in list(self._pending):
            t = self.tier_of(self._models[r.model][3])
            free = [s for s in self._slots if not s.busy and self._compatible(s, r)]
            if free:
                s = min(free, key=lambda s: s.tier)
                s.busy = True
                r.t_blocked = None
                return s, self._take_batch(s, r), False
            used = sum(s.bytes for s in self._slots)
            top = self.tier_of(max(m[3] for m in self._models))
            build = None
            if len(self._slots) < self.max_slots:     # the largest tier that fits as things stand
                for tt in sorted((x for x in self.tiers if t <= x <= top), reverse=True):
                    if used + int(self._estimate(tt, self.slot_points)) <= self.budget:
                        build = tt
                        break
            if build is None and self._make_room(int(self._estimate(t, self.slot_points))):
                build = t                             # its own tier, after retiring idle engines
            if build is not None:
                ids = [i for i, m in enumerate(self._models) if m[3] <= build]
                s = _Slot(build, ids, int(self._estimate(build, self.slot_points)))
                self._slots.append(s)
                r.t_blocked = None
                return s, self._take_batch(s, r), True
            if r.t_blocked is None:
                r.t_blocked = now
            if now - r.t_blocked > self.max_bypass_s:
                return None                 # hold later requests back until this one starts
        return None

    def _dispatch(self):
        workers = []
        while True:
            with self._cv:
                while True:
                    plan = self._plan() if self._pending else None
                    if plan is not None or (self._stop and not self._pending):
                        break
                    if self._stop and not any(s.busy for s in self._slots):
                        # closing, nothing running and nothing can start: fail the rest
                        for r in self._pending:
                            r.future.set_exception(RuntimeError("server closed before the request could start"))
                        self._pending.clear()
                        break
                    # re-plan when a slot frees, a request or model arrives, or a
                    # blocked request's bypass time runs out
                    self._cv.wait(timeout=0.05 if self._pending else None)
                if plan is None:
                    break
            t = threading.Thread(target=self._run, args=plan, daemon=True)
            t.start()
            workers.append(t)
            workers = [w for w in workers if w.is_alive()]
        for w in workers:
            w.join()

    # -- engines -----------------------------------------------------------------
    def _build(self, s: _Slot):
        ms = [self._models[i] for i in s.ids]
        e = self._factory([m[0] for m in ms], [m[1] for m in ms], [m[2] for m in ms], self.slot_points)
        actual = int(e.info().get("device_bytes", s.bytes) or s.bytes)
        with self._cv:
            s.engine = e
            s.bytes = actual
            self.engines_built += 1

    def _close_engine(self, s: _Slot):
        if s.engine is not None:
            try:
                self._retired_launches += int(s.engine.info().get("launches", 0))
            except Exception:
                pass
            close = getattr(s.engine, "close", None)
            if close:
                close()

    def _retire(self, s: _Slot):
        self._close_engine(s)
        s.engine = None
        self.engines_retired += 1

    def _run(self, s: _Slot, batch: list[Request], build: bool):
        t0 = time.perf_counter()
        try:
            if build:
                self._build(s)
            pm = np.concatenate([np.full(r.npts, s.local[r.model], np.int32) for r in batch])
            k = np.concatenate([r.kpts for r in batch])
            om = np.concatenate([r.omega for r in batch])
            et = np.concatenate([np.full(r.npts, r.eta) for r in batch])
            for r in batch:
                r.t_start = t0
            out = s.engine.run(pm, k, om, et, tol=self.tol, itermax=self.itermax,
                               divide_by_pi=self.divide_by_pi)
            t1 = time.perf_counter()
            with self._cv:
                self.batches.append((s.tier, int(len(pm))))
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
            if build and s.engine is None:          # the engine could not be built: drop its slot
                with self._cv:
                    if s in self._slots:
                        self._slots.remove(s)
        finally:
            with self._cv:
                s.busy = False
                s.last_used = time.perf_counter()
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
