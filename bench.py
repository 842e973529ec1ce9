#!/usr/bin/env python
"""Surface-GF (k, omega) solves/s on GB300 for WannierTools' surface-state path.

Default run (no flags): the Fermi-arc plane of a seeded synthetic TaAs-sized
model, Num_wann = 56, Np = 2 (Ndim = 112), a 201 x 201 k-plane over the full
surface BZ at omega = 0 with eta = 1e-3 eV, reference convergence settings
(tol = the 1e-16 single-precision literal, itermax = 100).  A step is one pass
of the hot path (Fourier sum + decimation + spectral sums) over a slab of B
consecutive k points of the plane; successive steps walk the plane.  The line
reports the all-FP64 form as `value` and the mixed (split-BF16 tensor-core)
form beside it, and carries a `configs` object with the other workloads, each
run for a bounded number of steps stated inside it:

  plane    the whole 201 x 201 plane of the default workload in one public-API
           call per form (host buffers), and the two forms' agreement over every
           one of its 40 401 points
  ss_n264  the k-path x omega spectrum at Ndim 264 (Num_wann 88, Np 3), 301 k x
           501 omega in [-0.5, 0.5] eV, eta 1e-3 eV: both forms, e2e, errors
  uneven4  four models of Ndim 16 / 40 / 112 / 264 interleaved in one persistent
           launch per step, eta log-uniform in [1e-4, 1e-2] eV: both forms
  serve8   the continuous-batching request loop over 8 models (Ndim 8..300):
           the mixed form at three Poisson rates of 200 requests each (p50 /
           p99 latency), and the FP64 form's saturated throughput

Arms:
  (default)          the GPU path.  `value`: device-resident inputs, timed with
                     CUDA events on the launching stream; `e2e`: the host-buffer
                     C-ABI call wtg_surface_spectrum (pinned k list in, dos out);
                     `cpu_baseline`: the CPU oracle on a bounded sample.
  --impl reference   the CPU oracle (numpy + LAPACK restatement of the
                     reference, one process per host core) on the same config.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "surface-GF (k,omega) solves/s"
NAMES = ("dos_l", "dos_r", "dos_bulk")


def _measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


MEASURED_PEAKS = _measured_peaks()
EV2HARTREE = 1.0 / 27.211385

WORKLOADS = {
    # the Fermi-arc plane (SurfaceDOSkk): one omega per k, /pi sums
    "arc_n112": dict(nw=56, np_=2, seed=2024, nk1=201, nk2=201, omega_ev=[0.0], eta_ev=1e-3,
                     divide_by_pi=True, tol=None, cpu_per_core=12, ref_per_core=4,
                     desc="SurfaceDOSkk Fermi-arc plane, synthetic Num_wann=56 Np=2 (Ndim=112), "
                          "201x201 k-plane, omega=0, eta=1e-3 eV"),
    # the k-path x omega spectrum (surfstat): 101 k x 201 omega, eta 1e-2 eV, tol 1e-10
    "ss_n40": dict(nw=20, np_=2, seed=2023, nk1=101, nk2=None, omega_ev=None, eta_ev=1e-2,
                   divide_by_pi=False, tol=1e-10, cpu_per_core=1, ref_per_core=1,
                   omega_range=(-1.0, 1.0), nomega=201,
                   desc="surfstat k-path x omega, synthetic Num_wann=20 Np=2 (Ndim=40), "
                        "101 k x 201 omega in [-1,1] eV, eta=1e-2 eV, tol=1e-10"),
    # four models of Ndim 16, 40, 112, 264 interleaved in one persistent launch per step; each
    # model has 4096 random (k, omega) points, eta log-uniform in [1e-4, 1e-2] eV; a step is 256
    # points of each model (the next slice of the 4 x 4096 set)
    "uneven4": dict(kind="uneven", shapes=[(8, 2), (20, 2), (56, 2), (88, 3)], seed=2027,
                    per_model=4096, step_per_model=256, cpu_per_model=16,
                    desc="uneven batch: synthetic models of Ndim 16/40/112/264 (Num_wann/Np "
                         "8/2, 20/2, 56/2, 88/3) interleaved in one persistent launch, 4096 "
                         "random (k,omega) each, eta log-uniform [1e-4,1e-2] eV"),
    # request loop: 8 models (Ndim 8..300), Poisson arrivals, requests of 50-400 points
    "serve8": dict(kind="serve", shapes=[(8, 1), (16, 2), (30, 2), (40, 3), (56, 2), (75, 2),
                                         (88, 3), (150, 2)], seed=2028, requests=200,
                   rates=(3.0, 6.0, 12.0), fp64_requests=16, slot_points=512, slots=4,
                   desc="serving loop: 8 synthetic models Num_wann 8..150, Np 1..3 (Ndim 8..300), "
                        "Poisson requests of 50-400 (k,omega) points, random omega windows in "
                        "[-1,1] eV, eta log-uniform [1e-3,1e-2] eV"),
    # the large k-path x omega spectrum: 301 k x 501 omega at Ndim 264; three k points
    # (1503 solves = 9.9 waves of one solve per SM) per step: two k points (6.6 waves) left
    # 41 % of the SMs idle in the last wave, 5 % of the step, which the whole 150 801-solve
    # configuration does not have; a strided subset of omegas in the CPU sample
    "ss_n264": dict(nw=88, np_=3, seed=2026, nk1=301, nk2=None, omega_ev=None, eta_ev=1e-3,
                    divide_by_pi=False, tol=None, cpu_per_core=1, ref_per_core=1,
                    omega_range=(-0.5, 0.5), nomega=501, step_k=3, cpu_omegas=6,
                    desc="surfstat k-path x omega, synthetic Num_wann=88 Np=3 (Ndim=264), "
                         "301 k x 501 omega in [-0.5,0.5] eV, eta=1e-3 eV"),
}

# bounded runs of the other workloads inside the default line's `configs`
CONFIG_RUNS = {
    "ss_n264": dict(steps={"fp64": 1, "mixed": 2}, warmup=1, e2e_steps=1, cpu_k=16),
    "uneven4": dict(steps=2, warmup=2),
}


def workload_points(wl: dict):
    """(k list (nk,2), omega list (Hartree)) of a workload."""
    import numpy as np
    from wannier_tools_gb300.api import kpath_slab, kplane_slab
    if wl["nk2"] is not None:
        _, _, k = kplane_slab(wl["nk1"], wl["nk2"], (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
        om = np.asarray(wl["omega_ev"]) * EV2HARTREE
    else:
        k = kpath_slab([((-0.5, 0.0), (0.5, 0.0))], wl["nk1"])
        om = np.linspace(wl["omega_range"][0], wl["omega_range"][1], wl["nomega"]) * EV2HARTREE
    return k, om


def cpu_omegas(wl: dict, om):
    """The omegas of each k point in the CPU sample: all of them, or an evenly
    strided subset where one k point's full omega list is too long for the
    bounded sample (Ndim 264)."""
    import numpy as np
    n = wl.get("cpu_omegas")
    if not n or n >= len(om):
        return om
    return om[np.linspace(0, len(om) - 1, n).round().astype(int)]


def orbitals(wl: dict):
    nw = wl["nw"]
    return list(range(1, nw + 1)), list(range(1, nw + 1))


# --- CPU oracle worker (spawned processes, one BLAS thread each) -------------

_MODEL_CACHE: dict = {}


def _cpu_model(wl):
    from wannier_tools_gb300 import synthetic
    key = (wl["nw"], wl["np_"], wl["seed"])
    if key not in _MODEL_CACHE:
        _MODEL_CACHE[key] = synthetic.make_model(wl["nw"], wl["np_"], seed=wl["seed"])
    return _MODEL_CACHE[key]


def _cpu_warm(wl):
    _cpu_model(wl)
    time.sleep(0.2)             # keep this worker busy so every worker gets one warm task
    return os.getpid()


def _cpu_worker(args):
    """Oracle spectrum of a k list (timed); with reordered=True the same steps in the
    oracle's other FP64 rounding order (the FP64 noise-floor probe, not timed)."""
    import numpy as np
    from oracle import wt_oracle as O
    wl, kpts, om, reordered = args
    m = _cpu_model(wl)
    top, bot = orbitals(wl)
    tol = wl["tol"] if wl["tol"] is not None else O.ACCURACY_REF
    t0 = time.perf_counter()
    r = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, np.asarray(kpts), np.asarray(om),
                           wl["eta_ev"] * EV2HARTREE, top, bot,
                           scale=(1.0 / O.PI_REF if wl["divide_by_pi"] else 1.0), accuracy=tol,
                           reordered=reordered)
    return time.perf_counter() - t0, {k: r[k] for k in NAMES}


def cpu_pool(ncores: int):
    import multiprocessing as mp
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    return mp.get_context("spawn").Pool(ncores)


def cpu_sample_rate(pool, ncores: int, wl: dict, per_core: int, offset: int = 0, nks: int = 0):
    """Solves/s of the oracle over ncores * per_core (or nks) k points of the
    workload, each with all of its sample omegas (one Fourier sum per k, as the
    reference's loops do)."""
    import numpy as np
    pool.map(_cpu_warm, [wl] * ncores, chunksize=1)
    k, om = workload_points(wl)
    om = cpu_omegas(wl, om)
    nks = nks or ncores * per_core
    idx = (offset + np.arange(nks) * max(1, len(k) // nks)) % len(k)
    tasks = [(wl, k[[i]], om, False) for i in idx]
    t0 = time.perf_counter()
    res = pool.map(_cpu_worker, tasks, chunksize=1)
    wall = time.perf_counter() - t0
    npts = nks * len(om)
    ref = {name: np.concatenate([r[1][name] for r in res]) for name in NAMES}
    return npts / wall, wall, npts, k[idx], ref, om


def reference_spread(pool, wl, k_sample, om_sample, ref):
    """Max relative distance of the oracle's reordered FP64 evaluation from the
    oracle on the sample: how far two valid FP64 evaluations of the reference's
    algorithm lie apart there."""
    import numpy as np
    res = pool.map(_cpu_worker, [(wl, k_sample[[i]], om_sample, True) for i in range(len(k_sample))],
                   chunksize=1)
    out = {}
    for name in NAMES:
        alt = np.concatenate([r[1][name] for r in res])
        out[name] = float(np.max(np.abs(alt - ref[name]) / np.abs(ref[name])))
    return out


def max_rel(got, ref):
    import numpy as np
    return {name: float(np.max(np.abs(np.asarray(got[name]).ravel() - np.asarray(ref[name]).ravel())
                               / np.abs(np.asarray(ref[name]).ravel()))) for name in NAMES}


# --- clocks during the timed region -------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        # the raw samples (the JSON line carries their summary); WTG_CLOCKS_DIR keeps them
        clock_dir = Path(os.environ.get("WTG_CLOCKS_DIR") or tempfile.gettempdir())
        self.path = clock_dir / f"clocks_bench_{os.getpid()}_{id(self)}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sms.append(float(p[1]))
                maxs.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sms) if sms else None,
                "sm_max_mhz": max(maxs) if maxs else None, "reasons": sorted(reasons),
                "samples": len(sms)}


# --- arms ---------------------------------------------------------------------

def dist_setup(backend: str):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank, local


class SpectrumRun:
    """One spectrum workload on the GPU: the model resident, k slabs of B points,
    device inputs/outputs for the CUDA-event timing, pinned host buffers for the
    host-buffer (e2e) call."""

    def __init__(self, wl, dev, ws=1, rank=0, batch=0, nslabs=8, nomega=0):
        import numpy as np
        import torch

        import wannier_tools_gb300 as w
        from wannier_tools_gb300 import api
        self.wl, self.dev, self.ws, self.rank = wl, dev, ws, rank
        self.m = w.make_model(wl["nw"], wl["np_"], seed=wl["seed"])
        self.model = w.Model.from_surface_model(self.m)
        self.k_all, self.om = workload_points(wl)
        if 0 < nomega < len(self.om):        # a smaller step: evenly strided omegas of the list
            self.om = self.om[np.linspace(0, len(self.om) - 1, nomega).round().astype(int)]
        self.top, self.bot = orbitals(wl)
        self.nomega = len(self.om)
        nsm = torch.cuda.get_device_properties(dev).multi_processor_count
        self.B = batch or wl.get("step_k") or (nsm * 8 if self.nomega == 1 else max(1, (nsm * 8 * 4) // self.nomega))
        self.tol = wl["tol"] if wl["tol"] is not None else api.ACCURACY_REF
        self.eta = wl["eta_ev"] * EV2HARTREE
        self.n_slabs = (len(self.k_all) + self.B - 1) // self.B
        self.n3 = float(self.m.ndim) ** 3
        self.stream = torch.cuda.current_stream(dev)
        self.d_om = torch.tensor(self.om, dtype=torch.float64, device=dev)
        self.slabs = [torch.tensor(np.ascontiguousarray(self.slab(i).T), dtype=torch.float64, device=dev)
                      for i in range(nslabs)]
        self.outs = [torch.empty((self.nomega, self.B), dtype=torch.float64, device=dev) for _ in range(3)]
        self.d_it = [torch.empty((self.nomega, self.B), dtype=torch.int32, device=dev) for _ in range(nslabs)]
        self.d_st = [torch.empty((self.nomega, self.B), dtype=torch.uint8, device=dev) for _ in range(nslabs)]
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)    # > L2 (126 MiB)
        self.kpin = [torch.empty((2, self.B), dtype=torch.float64).pin_memory().numpy() for _ in range(nslabs)]
        for i in range(nslabs):
            self.kpin[i][:] = self.slab(i).T
        n = self.B * self.nomega
        self.hout = {name: torch.empty(n, dtype=torch.float64).pin_memory().numpy() for name in NAMES}
        self.hout["iters"] = torch.empty(n, dtype=torch.int32).pin_memory().numpy()
        self.hout["status"] = torch.empty(n, dtype=torch.uint8).pin_memory().numpy()

    def slab(self, step):
        import numpy as np
        s = (step * self.ws + self.rank) % self.n_slabs
        idx = (np.arange(self.B) + s * self.B) % len(self.k_all)
        return self.k_all[idx]

    def measure(self, prec, steps, warmup, e2e_steps):
        """value: CUDA events over `steps` device-buffer steps (after `warmup`);
        e2e: wall clock over `e2e_steps` host-buffer calls."""
        import numpy as np
        import torch
        wl, model, dev, stream = self.wl, self.model, self.dev, self.stream
        nsl = len(self.slabs)

        def step(i):
            self.flush.zero_()
            j = i % nsl
            model.surface_spectrum_device(self.slabs[j], self.d_om, self.eta, self.top, self.bot,
                                          self.outs[0], self.outs[1], self.outs[2], self.d_it[j],
                                          self.d_st[j], tol=self.tol, divide_by_pi=wl["divide_by_pi"],
                                          precision=prec, stream=stream.cuda_stream)

        for i in range(warmup):
            step(i)
        torch.cuda.synchronize(dev)
        if self.ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        model.profile(True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(dev.index or 0) as clk:
            e0.record(stream)
            for i in range(warmup, warmup + steps):
                step(i)
            e1.record(stream)
            torch.cuda.synchronize(dev)
        if self.ws > 1:
            torch.distributed.barrier()
        ms = e0.elapsed_time(e1)
        prof = model.profile_read()
        model.profile(False)
        timed = [(i % nsl) for i in range(warmup, warmup + steps)]
        its = np.concatenate([self.d_it[j].cpu().numpy().ravel() for j in timed])
        st = np.concatenate([self.d_st[j].cpu().numpy().ravel() for j in timed])
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        if self.ws > 1:
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_max = float(t.item())
        solves = self.ws * steps * self.B * self.nomega
        # e2e through the host-buffer C ABI (pinned k list in, dos/iters/status out)
        model.surface_spectrum(None, self.om, self.eta, self.top, self.bot, tol=self.tol,
                               divide_by_pi=wl["divide_by_pi"], precision=prec, kcol=self.kpin[0],
                               out=self.hout)      # warm the host path
        if self.ws > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for i in range(e2e_steps):
            self.flush.zero_()
            torch.cuda.synchronize(dev)
            model.surface_spectrum(None, self.om, self.eta, self.top, self.bot, tol=self.tol,
                                   divide_by_pi=wl["divide_by_pi"], precision=prec,
                                   kcol=self.kpin[(warmup + i) % nsl], out=self.hout)
        te = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device=dev)
        if self.ws > 1:
            torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
        return {"value": solves / (ms_max / 1e3), "ms": ms_max, "steps": steps,
                "e2e": self.ws * e2e_steps * self.B * self.nomega / float(te.item()),
                "e2e_steps": e2e_steps, "prof": prof, "its": its, "st": st, "clocks": clk.summary()}

    def e2e_bytes(self):
        return {"h2d_bytes_per_step": self.B * 2 * 8 + self.nomega * 8,
                "d2h_bytes_per_step": self.B * self.nomega * (3 * 8 + 4 + 1)}

    def roofline(self, f, r, peaks):
        """Roofline of the decimation kernel from this run's live CUDA-event times.
        Work is algorithmic: (56 it + 24) Ndim^3 flops per solve, it = the FP64 form's
        iteration count of each point (both forms iterate alike within +-1)."""
        import numpy as np
        prof, its = r["prof"], r["its"]
        launch_ms = prof["decim_ms"] / max(1, prof["decim_launches"])
        alg = float(((56.0 * its + 24.0) * self.n3).sum())
        ach = alg / (prof["decim_ms"] / 1e3) / 1e12 if prof["decim_ms"] > 0 else None
        if f == "fp64":
            peak = max(peaks["dfma"], peaks["dmma"])
            traffic = traffic_per_solve(self.wl_name())
            return {"bound": "fp64", "kernel": "k_decimate_fp64", "achieved": ach, "peak": peak,
                    "unit": "TFLOP/s", "frac": (ach / peak) if ach else None,
                    "traffic": (traffic * self.B * self.nomega) if traffic else None,
                    "traffic_unit": "bytes per launch",
                    "peak_source": "the faster FP64 path measured live on this GPU: DFMA "
                                   f"{peaks['dfma']:.3f} TFLOP/s (wtg_probe_fp64_peak), DMMA "
                                   f"{peaks['dmma']:.3f} TFLOP/s (mma.sync m8n8k4 .f64, "
                                   "wtg_probe_dmma_peak)",
                    "dfma_peak": peaks["dfma"], "dmma_peak": peaks["dmma"], "launch_ms": launch_ms,
                    "work": "(56*it+24)*Ndim^3 flops per solve, it = FP64 iterations"}
        m = self.m
        npad = (m.ndim + 7) // 8 * 8
        nch = (m.ndim + 15) // 16
        nrb = (m.ndim + 127) // 128
        # BF16 MMA flops issued by one 7-digit complex product: row blocks of 128 x 2
        # components x K chunks x 28 slice pairs x 2 real products x 2*128*16 flops per
        # output column over Ndim columns rounded up to 8; 7 such products per iteration (six loop products
        # and the refinement's residual), the 4-digit correction (10 pairs) as 10/28 of one
        per_prod = nrb * 2 * nch * 56 * 2.0 * 128 * 16 * npad
        issued = float(((7.0 + 10.0 / 28.0) * its * per_prod).sum())
        iss = issued / (prof["decim_ms"] / 1e3) / 1e12 if prof["decim_ms"] > 0 else None
        peak = MEASURED_PEAKS.get("bf16_tflops")
        return {"bound": "tensor", "kernel": "k_decimate_mixed", "achieved": ach, "peak": peak,
                "unit": "TFLOP/s", "frac": (ach / peak) if (ach and peak) else None, "traffic": None,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)", "launch_ms": launch_ms,
                "work": "(56*it+24)*Ndim^3 FP64-equivalent flops per solve (algorithmic)",
                "issued_bf16_tflops": iss, "issued_frac": (iss / peak) if (iss and peak) else None,
                "issued_work": "BF16 MMA flops issued: per iteration 7 products of 28 slice pairs and "
                               "one of 10, each ceil(Ndim/128) row blocks x 2 components x "
                               "ceil(Ndim/16) K chunks x 2*128*16 flops per column x Ndim columns rounded up to 8",
                "vs_fp64_peak": (ach / max(peaks["dfma"], peaks["dmma"])) if ach else None}

    def wl_name(self):
        for k, v in WORKLOADS.items():
            if v is self.wl:
                return k
        return ""

    def close(self):
        self.model.close()


def fp64_peaks():
    from wannier_tools_gb300 import api
    return {"dfma": api.fp64_peak_tflops(), "dmma": api.dmma_peak_tflops()}


def form_summary(run, f, r, peaks, errors=None):
    return {"value": r["value"], "e2e": r["e2e"], "ms_per_step": r["ms"] / r["steps"],
            "steps": r["steps"], "e2e_steps": r["e2e_steps"],
            "gpu_launches": r["prof"]["launches"], "roofline": run.roofline(f, r, peaks),
            "mean_iterations": float(r["its"].mean()),
            "status_flagged_points": int((r["st"] != 0).sum()),
            "max_rel_err_vs_fp64_oracle": errors, "clocks": r["clocks"]}


def run_gpu(args):
    import torch

    import wannier_tools_gb300 as w
    from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED

    wl = WORKLOADS[args.workload]
    ws, rank, local = dist_setup("nccl")
    pool = None
    ncores = os.cpu_count() or 1
    if rank == 0 and not args.no_cpu_baseline:
        pool = cpu_pool(ncores)               # spawn before the first GPU call
    torch.cuda.set_device(local)
    w.build()
    dev = torch.device("cuda", local)
    nsteps = args.warmup + args.steps
    run = SpectrumRun(wl, dev, ws, rank, args.batch, nslabs=nsteps, nomega=args.nomega)
    precs = {"fp64": PREC_FP64, "mixed": PREC_MIXED}
    primary = args.precision
    forms = [primary] + ([] if args.only else [p for p in ("fp64", "mixed") if p != primary])
    e2e_steps = min(args.steps, args.e2e_steps)
    res = {f: run.measure(precs[f], args.steps, args.warmup, e2e_steps) for f in forms}
    peaks = fp64_peaks()

    cpu = None
    errors = {}
    spread = None
    if pool is not None:
        per_core = args.cpu_sample_per_core
        rate, wall, npts, k_sample, oracle_ref, om_sample = cpu_sample_rate(pool, ncores, wl, per_core)
        cpu = {"value": rate, "unit": "solves/s", "cores": ncores, "kind": "port",
               "sample": f"{npts} (k,omega) solves: {ncores * per_core} k points of the same "
                         f"workload x {len(om_sample)} of their {run.nomega} omegas, {ncores} spawned "
                         f"processes x 1 OpenBLAS thread, {wall:.1f} s wall"}
        spread = reference_spread(pool, wl, k_sample, om_sample, oracle_ref)
        for f in forms:   # max relative error of each form against the FP64 oracle on that sample
            g = run.model.surface_spectrum(k_sample, om_sample, run.eta, run.top, run.bot, tol=run.tol,
                                           divide_by_pi=wl["divide_by_pi"], precision=precs[f])
            errors[f] = max_rel(g, oracle_ref)
            errors[f]["points"] = int(npts)
            if f == "fp64":
                errors[f]["reference_fp64_spread"] = spread

    configs = None
    if rank == 0 and ws == 1 and args.workload == "arc_n112" and not args.no_configs:
        configs = {}
        for name, fn in (("plane", lambda: plane_config(run)),
                         ("ss_n264", lambda: ss_n264_config(dev, pool, ncores, peaks)),
                         ("uneven4", lambda: uneven_config(pool, ncores)),
                         ("serve8", serve_config)):
            t0 = time.perf_counter()
            try:
                configs[name] = fn()
            except Exception as e:      # one workload's failure must not lose the line
                configs[name] = {"error": f"{type(e).__name__}: {e}"}
            configs[name]["run_s"] = time.perf_counter() - t0

    if rank == 0:
        r = res[primary]
        line = {
            "metric": METRIC, "value": r["value"], "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["desc"], "k_points_per_step": run.B, "omegas_per_k": run.nomega,
                       "ndim": run.m.ndim, "precision": primary,
                       "parallelism": f"replicas x{ws} (k slabs)",
                       "l2": "flushed between steps (256 MiB write)",
                       "status_flagged_points": int((r["st"] != 0).sum()),
                       "mean_iterations": float(r["its"].mean())},
            "e2e": {"value": r["e2e"], "unit": "solves/s", "steps": e2e_steps, **run.e2e_bytes()},
            "gpu_launches": r["prof"]["launches"],
            "roofline": run.roofline(primary, r, peaks),
            "fourier_ms_per_step": r["prof"]["fourier_ms"] / args.steps,
            "clocks": r["clocks"],
            "cpu_baseline": cpu,
            "max_rel_err_vs_fp64_oracle": errors.get(primary),
        }
        for f in forms[1:]:
            o = res[f]
            line[f] = form_summary(run, f, o, peaks, errors.get(f))
            line[f]["speedup_vs_" + primary] = o["value"] / r["value"]
            line[f]["e2e_speedup_vs_" + primary] = o["e2e"] / r["e2e"]
        if configs is not None:
            line["configs"] = configs
        print(json.dumps(line))
    run.close()
    if pool is not None:
        pool.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def plane_config(run):
    """The whole configuration end to end: every k point of the workload (all 40 401 points of
    the 201 x 201 arc plane) in one public-API call per form, host k list in and host DOS out,
    and the two forms' agreement over every point of the plane (a full-size check beside the
    sampled oracle errors of the line)."""
    import numpy as np
    import torch

    from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED
    wl, dev = run.wl, run.dev
    npts = len(run.k_all) * run.nomega
    out = {"workload": wl["desc"], "points": npts,
           "timing": "wall clock around one surface_spectrum call over every k point (host k "
                     "list in, host dos_l / dos_r / dos_bulk / iters / status out)"}
    res = {}
    for f, prec in (("mixed", PREC_MIXED), ("fp64", PREC_FP64)):
        run.flush.zero_()
        torch.cuda.synchronize(dev)
        with ClockSampler(dev.index or 0) as clk:
            t0 = time.perf_counter()
            g = run.model.surface_spectrum(run.k_all, run.om, run.eta, run.top, run.bot, tol=run.tol,
                                           divide_by_pi=wl["divide_by_pi"], precision=prec)
            dt = time.perf_counter() - t0
        res[f] = g
        out[f] = {"value": npts / dt, "unit": "solves/s", "wall_s": dt,
                  "mean_iterations": float(g["iters"].mean()),
                  "status_flagged_points": int((g["status"] != 0).sum()), "clocks": clk.summary()}
    out["mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["mixed_max_rel_diff_vs_fp64"] = max_rel(res["mixed"], res["fp64"])
    out["fp64_sums"] = {name: float(np.sum(res["fp64"][name])) for name in NAMES}
    return out


def ss_n264_config(dev, pool, ncores, peaks):
    """The Ndim-264 k-path x omega spectrum, both forms, bounded steps (CONFIG_RUNS)."""
    import numpy as np

    from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED
    wl = WORKLOADS["ss_n264"]
    cr = CONFIG_RUNS["ss_n264"]
    nsl = cr["warmup"] + max(cr["steps"].values())
    run = SpectrumRun(wl, dev, nslabs=nsl)
    precs = {"fp64": PREC_FP64, "mixed": PREC_MIXED}
    res = {f: run.measure(precs[f], cr["steps"][f], cr["warmup"], cr["e2e_steps"]) for f in ("fp64", "mixed")}
    out = {"workload": wl["desc"], "k_points_per_step": run.B, "omegas_per_k": run.nomega,
           "warmup": cr["warmup"], "l2": "flushed between steps (256 MiB write)"}
    errors, spread, cpu = {}, None, None
    if pool is not None:
        rate, wall, npts, k_sample, ref, om_sample = cpu_sample_rate(pool, ncores, wl, 1, nks=cr["cpu_k"])
        spread = reference_spread(pool, wl, k_sample, om_sample, ref)
        cpu = {"value": rate, "unit": "solves/s", "cores": ncores, "kind": "port",
               "sample": f"{npts} solves: {cr['cpu_k']} k points x {len(om_sample)} strided omegas"}
        for f in ("fp64", "mixed"):
            g = run.model.surface_spectrum(k_sample, om_sample, run.eta, run.top, run.bot, tol=run.tol,
                                           precision=precs[f])
            errors[f] = max_rel(g, ref)
            errors[f]["points"] = int(npts)
        errors["fp64"]["reference_fp64_spread"] = spread
    for f in ("fp64", "mixed"):
        out[f] = form_summary(run, f, res[f], peaks, errors.get(f))
        out[f]["e2e_bytes"] = run.e2e_bytes()
    out["mixed_vs_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    out["mixed_vs_fp64_e2e"] = res["mixed"]["e2e"] / res["fp64"]["e2e"]
    out["cpu_oracle"] = cpu
    run.close()
    return out


# --- uneven batch ---------------------------------------------------------------

def _uneven_points(wl):
    import numpy as np
    rng = np.random.default_rng(wl["seed"])
    nm, per = len(wl["shapes"]), wl["per_model"]
    k = rng.uniform(-0.5, 0.5, (nm, per, 2))
    om = rng.uniform(-1.0, 1.0, (nm, per)) * EV2HARTREE
    eta = np.exp(rng.uniform(np.log(1e-4), np.log(1e-2), (nm, per))) * EV2HARTREE
    return k, om, eta


def _uneven_step(wl, step):
    """Points of one step: the step-th slice of step_per_model points of every model, interleaved."""
    import numpy as np
    k, om, eta = _uneven_points(wl)
    nm, sp, per = len(wl["shapes"]), wl["step_per_model"], wl["per_model"]
    idx = (np.arange(sp) + step * sp) % per
    pm = np.tile(np.arange(nm, dtype=np.int32), sp)
    ii = np.repeat(idx, nm)
    return pm, k[pm, ii], om[pm, ii], eta[pm, ii]


def _uneven_cpu_worker(args):
    import numpy as np
    from oracle import wt_oracle as O
    from wannier_tools_gb300 import synthetic
    (nw, np_, seed), kk, om, eta = args
    m = synthetic.make_model(nw, np_, seed=seed)
    allorb = list(range(1, nw + 1))
    t0 = time.perf_counter()
    r = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, np.asarray([kk]), np.asarray([om]),
                           eta, allorb, allorb)
    return time.perf_counter() - t0, (float(r["dos_l"][0, 0]), float(r["dos_r"][0, 0]),
                                      float(r["dos_bulk"][0, 0]))


def uneven_measure(wl, forms, steps, warmup, pool, ncores):
    """Each step: one persistent launch over the next 256 points of every model, through
    wtg_engine_run (host inputs and outputs; graph-replayed)."""
    import numpy as np
    import torch

    import wannier_tools_gb300 as w
    from wannier_tools_gb300 import api
    from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED
    ms = [w.make_model(nw, np_, seed=wl["seed"] + i) for i, (nw, np_) in enumerate(wl["shapes"])]
    gs = [w.Model.from_surface_model(m) for m in ms]
    tops = [list(range(1, m.nw + 1)) for m in ms]
    npts = len(wl["shapes"]) * wl["step_per_model"]
    precs = {"fp64": PREC_FP64, "mixed": PREC_MIXED}
    res = {}
    for f in forms:
        with api.Engine(gs, tops, tops, precision=precs[f], max_points=npts) as eng:
            for i in range(warmup):
                eng.run(*_uneven_step(wl, i))
            todo = [_uneven_step(wl, warmup + i) for i in range(steps)]
            l0 = eng.info()["launches"]
            torch.cuda.synchronize()
            with ClockSampler(0) as clk:
                t0 = time.perf_counter()
                outs = [eng.run(*st) for st in todo]
                dt = time.perf_counter() - t0
            n3 = np.array([float(m.ndim) ** 3 for m in ms])
            its = np.concatenate([o["iters"] for o in outs])
            pms = np.concatenate([st[0] for st in todo])
            res[f] = {"value": len(pms) / dt, "ms": 1e3 * dt / steps, "clocks": clk.summary(),
                      "its": its, "flagged": int(sum((o["status"] != 0).sum() for o in outs)),
                      "fp64_flops": float(((56.0 * its + 24.0) * n3[pms]).sum()), "dt": dt,
                      "launches": eng.info()["launches"] - l0, "first": (todo[0], outs[0])}
    cpu, errs = None, {}
    if pool is not None:
        # bounded oracle sample: cpu_per_model points of each model from the first timed step
        (pm, k, om, eta), _ = res[forms[0]]["first"]
        sel = np.concatenate([np.where(pm == i)[0][:wl["cpu_per_model"]] for i in range(len(ms))])
        tasks = [((wl["shapes"][pm[j]][0], wl["shapes"][pm[j]][1], wl["seed"] + int(pm[j])), k[j],
                  om[j], eta[j]) for j in sel]
        pool.map(_cpu_warm, [WORKLOADS["ss_n40"]] * ncores, chunksize=1)
        t0 = time.perf_counter()
        rs = pool.map(_uneven_cpu_worker, tasks, chunksize=1)
        wall = time.perf_counter() - t0
        cpu = {"value": len(sel) / wall, "unit": "solves/s", "cores": ncores, "kind": "port",
               "sample": f"{len(sel)} points ({wl['cpu_per_model']} per model) of the first timed "
                         f"step, {ncores} spawned processes x 1 OpenBLAS thread, {wall:.1f} s wall"}
        ref = np.array([r[1] for r in rs])
        for f in forms:
            o = res[f]["first"][1]
            got = np.stack([o["dos_l"][sel], o["dos_r"][sel], o["dos_bulk"][sel]], 1)
            e = np.abs(got - ref) / np.abs(ref)
            errs[f] = {"dos_l": float(e[:, 0].max()), "dos_r": float(e[:, 1].max()),
                       "dos_bulk": float(e[:, 2].max()), "points": int(len(sel))}
    for g in gs:
        g.close()
    return res, cpu, errs, npts


def uneven_config(pool, ncores):
    wl = WORKLOADS["uneven4"]
    cr = CONFIG_RUNS["uneven4"]
    res, cpu, errs, npts = uneven_measure(wl, ["fp64", "mixed"], cr["steps"], cr["warmup"], pool, ncores)
    out = {"workload": wl["desc"], "points_per_step": npts, "steps": cr["steps"], "warmup": cr["warmup"],
           "timing": "wall clock around wtg_engine_run (host inputs and outputs, graph-replayed)",
           "cpu_oracle": cpu}
    for f in ("fp64", "mixed"):
        o = res[f]
        out[f] = {"value": o["value"], "e2e": o["value"], "ms_per_step": o["ms"],
                  "fp64_equivalent_tflops": o["fp64_flops"] / o["dt"] / 1e12,
                  "mean_iterations": float(o["its"].mean()), "status_flagged_points": o["flagged"],
                  "gpu_launches": o["launches"], "max_rel_err_vs_fp64_oracle": errs.get(f),
                  "clocks": o["clocks"]}
    out["mixed_vs_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    return out


def run_uneven(args):
    """One persistent launch per step over points of four models of different Ndim."""
    import torch

    import wannier_tools_gb300 as w
    wl = WORKLOADS[args.workload]
    ncores = os.cpu_count() or 1
    pool = None if args.no_cpu_baseline else cpu_pool(ncores)
    w.build()
    torch.cuda.set_device(0)
    forms = [args.precision] + ([] if args.only else [f for f in ("fp64", "mixed") if f != args.precision])
    res, cpu, errs, npts = uneven_measure(wl, forms, args.steps, args.warmup, pool, ncores)
    if pool is not None:
        pool.close()
    r = res[forms[0]]
    line = {"metric": METRIC, "value": r["value"], "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["desc"], "points_per_step": npts, "precision": forms[0],
                       "launch": "one persistent k_batch launch per step, points in cost order",
                       "timing": "wall clock around wtg_engine_run (host inputs, host outputs)",
                       "l2": "inputs larger than L2: 152 workspaces of 9-11 x 264^2 complex",
                       "mean_iterations": float(r["its"].mean()), "status_flagged_points": r["flagged"]},
            "e2e": {"value": r["value"], "unit": "solves/s", "h2d_bytes_per_step": npts * 40,
                    "d2h_bytes_per_step": npts * 29},
            "gpu_launches": r["launches"],
            "fp64_equivalent_tflops": r["fp64_flops"] / r["dt"] / 1e12,
            "clocks": r["clocks"], "cpu_baseline": cpu, "max_rel_err_vs_fp64_oracle": errs.get(forms[0])}
    for f in forms[1:]:
        o = res[f]
        line[f] = {"value": o["value"], "ms_per_step": o["ms"], "speedup_vs_" + forms[0]: o["value"] / r["value"],
                   "fp64_equivalent_tflops": o["fp64_flops"] / o["dt"] / 1e12,
                   "mean_iterations": float(o["its"].mean()), "status_flagged_points": o["flagged"],
                   "max_rel_err_vs_fp64_oracle": errs.get(f), "clocks": o["clocks"]}
    print(json.dumps(line))


# --- serving loop ---------------------------------------------------------------

def serve_measure(wl, prec, rates, requests, warm=3):
    """Poisson replays through the continuous-batching loop, one per rate."""
    import numpy as np
    import torch

    import wannier_tools_gb300 as w
    from wannier_tools_gb300.serving import SurfaceServer, poisson_requests, replay
    ms = [w.make_model(nw, np_, seed=wl["seed"] + i) for i, (nw, np_) in enumerate(wl["shapes"])]
    gs = [w.Model.from_surface_model(m) for m in ms]
    tops = [list(range(1, m.nw + 1)) for m in ms]
    sweep = []
    with SurfaceServer(gs, tops, tops, precision=prec, slot_points=wl["slot_points"],
                       max_slots=wl["slots"]) as srv:
        replay(srv, poisson_requests(np.random.default_rng(1), len(ms), 1e3, warm), EV2HARTREE)
        torch.cuda.synchronize()
        l0 = srv.launches()
        with ClockSampler(0) as clk:
            for i, rate in enumerate(rates):
                reqs = poisson_requests(np.random.default_rng(wl["seed"] + i), len(ms), rate, requests)
                rep = replay(srv, reqs, EV2HARTREE)
                rep.pop("results")
                rep["rate_per_s"] = rate
                sweep.append(rep)
        launches = srv.launches() - l0
        nslots = srv.engines_built
    for g in gs:
        g.close()
    return {"sweep": sweep, "clocks": clk.summary(), "launches": launches, "slots": nslots}


def serve_config():
    from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED
    wl = WORKLOADS["serve8"]
    mixed = serve_measure(wl, PREC_MIXED, wl["rates"], wl["requests"])
    # the FP64 form saturates near 1.2 requests/s: its throughput from one replay of
    # fp64_requests requests arriving at once (latency then is queueing, not reported)
    fp64 = serve_measure(wl, PREC_FP64, (1000.0,), wl["fp64_requests"])
    best = max(mixed["sweep"], key=lambda x: x["solves_per_s"])
    f = fp64["sweep"][0]
    return {"workload": wl["desc"], "engines_built": mixed["slots"], "max_engines": wl["slots"],
            "slot_points": wl["slot_points"],
            "timing": "wall clock from first arrival to last completion of each replay",
            "mixed": {"value": best["solves_per_s"], "requests_per_rate": wl["requests"],
                      "sweep": [{k: x[k] for k in ("rate_per_s", "requests", "points", "wall_s",
                                                   "solves_per_s", "p50_ms", "p99_ms", "flagged")}
                                for x in mixed["sweep"]],
                      "gpu_launches": mixed["launches"], "clocks": mixed["clocks"]},
            "fp64": {"value": f["solves_per_s"], "requests": f["requests"], "points": f["points"],
                     "wall_s": f["wall_s"], "arrival": "all at once (saturated)",
                     "gpu_launches": fp64["launches"], "clocks": fp64["clocks"]},
            "mixed_vs_fp64": best["solves_per_s"] / f["solves_per_s"]}


def run_serve(args):
    """Poisson request streams through the continuous-batching loop at swept rates."""
    import torch

    import wannier_tools_gb300 as w
    from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED
    wl = WORKLOADS[args.workload]
    w.build()
    torch.cuda.set_device(0)
    precs = {"fp64": PREC_FP64, "mixed": PREC_MIXED}
    forms = [args.precision] + ([] if args.only else [f for f in ("fp64", "mixed") if f != args.precision])
    rates = tuple(args.serve_rates) if args.serve_rates else wl["rates"]
    nreq = args.serve_requests or wl["requests"]
    out = {f: serve_measure(wl, precs[f], rates, nreq, warm=max(3, args.warmup)) for f in forms}
    r = out[forms[0]]
    best = max(r["sweep"], key=lambda x: x["solves_per_s"])
    line = {"metric": METRIC, "value": best["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
            "steps": len(r["sweep"]), "warmup": max(3, args.warmup),
            "ms_per_step": 1e3 * sum(x["wall_s"] for x in r["sweep"]) / len(r["sweep"]),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": wl["desc"], "precision": forms[0], "engines_built": r["slots"],
                       "max_engines": wl["slots"],
                       "slot_points": wl["slot_points"], "requests_per_rate": nreq,
                       "step": "one Poisson replay at one rate; value = best served solves/s",
                       "timing": "wall clock from first arrival to last completion"},
            "latency_ms": {"p50": best["p50_ms"], "p99": best["p99_ms"], "at_rate_per_s": best["rate_per_s"]},
            "sweep": r["sweep"],
            "e2e": {"value": best["solves_per_s"], "unit": "solves/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None},
            "gpu_launches": r["launches"], "clocks": r["clocks"], "cpu_baseline": None}
    for f in forms[1:]:
        o = out[f]
        ob = max(o["sweep"], key=lambda x: x["solves_per_s"])
        line[f] = {"value": ob["solves_per_s"], "latency_ms": {"p50": ob["p50_ms"], "p99": ob["p99_ms"],
                                                              "at_rate_per_s": ob["rate_per_s"]},
                   "sweep": o["sweep"], "clocks": o["clocks"]}
    print(json.dumps(line))


# --- reference arm ---------------------------------------------------------------

def traffic_per_solve(workload: str):
    """DRAM bytes per solve of the decimation kernel from the committed ncu
    summary (profiles/k_decimate_fp64_<workload>.md, line 'traffic_bytes_per_solve:')."""
    p = ROOT / "profiles" / f"k_decimate_fp64_{workload}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_solve:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def run_reference(args):
    wl = WORKLOADS[args.workload]
    ws, rank, _ = dist_setup("gloo")
    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    ncores = os.cpu_count() or 1
    pool = cpu_pool(ncores)
    per_core = args.ref_per_core
    for i in range(args.warmup):
        cpu_sample_rate(pool, ncores, wl, per_core, offset=i * 7919)
    total_pts, total_s = 0, 0.0
    for i in range(args.steps):
        _, wall, npts, _, _, om_s = cpu_sample_rate(pool, ncores, wl, per_core,
                                                    offset=(args.warmup + i) * 7919)
        total_pts += npts
        total_s += wall
    pool.close()
    nom_all = len(workload_points(wl)[1])
    om_desc = "all omegas" if len(om_s) == nom_all else f"{len(om_s)} of {nom_all} omegas"
    value = total_pts / total_s
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": wl["desc"], "precision": "fp64",
                       "sample_per_step": f"{ncores * per_core} k points x {om_desc}"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": ncores, "kind": "port",
                             "sample": f"{ncores * per_core} k points (x {om_desc}) per step spread "
                                       f"over the workload; numpy+OpenBLAS restatement of the reference "
                                       f"(the Fortran reference cannot be built here), one process "
                                       f"per core"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="arc_n112")
    ap.add_argument("--batch", type=int, default=0, help="k points per step (0 = 8 x SMs)")
    ap.add_argument("--nomega", type=int, default=0,
                    help="omegas per k point: this many evenly strided ones of the workload's list "
                         "(0 = all); with --batch, a smaller launch of the same kernel")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="default workload only: leave out the `configs` runs of the other workloads")
    ap.add_argument("--e2e-steps", type=int, default=5, help="host-buffer steps timed for e2e (<= --steps)")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64",
                    help="form reported as `value` (the other is reported beside it)")
    ap.add_argument("--only", action="store_true", help="time only the --precision form")
    ap.add_argument("--cpu-sample-per-core", type=int, default=0,
                    help="k points per host core in the cpu_baseline sample (0 = by workload)")
    ap.add_argument("--ref-per-core", type=int, default=0,
                    help="k points per host core per reference-arm step (0 = by workload)")
    ap.add_argument("--serve-rates", type=float, nargs="*", help="serve8: request rates (per s)")
    ap.add_argument("--serve-requests", type=int, default=0, help="serve8: requests per rate")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if wl.get("kind") in ("uneven", "serve"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched or "
                              "served form of this path; its CPU arm is timed on arc_n112/ss_n40/ss_n264"}))
            return
        if args.warmup < 3:
            ap.error("--warmup must be >= 3")
        (run_uneven if wl["kind"] == "uneven" else run_serve)(args)
        return
    if args.cpu_sample_per_core <= 0:
        args.cpu_sample_per_core = wl["cpu_per_core"]
    if args.ref_per_core <= 0:
        args.ref_per_core = wl["ref_per_core"]
    if args.warmup < 3 and args.impl == "ours":
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
