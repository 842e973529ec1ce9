"""Autotuner of the kernels' launch shapes: the tile table behind wtg_tile_set.

The tunable shape is, per Ndim,

* FP64 (per-model kernel, Ndim <= 119 where the inverse runs in shared memory):
  threads per CTA, 128, 256 or 512 (the GEMM's register rows per pass follow);
* mixed (split-BF16 products on the tensor cores): the output-column pass width,
  a multiple of 8 up to the tensor-memory limit (40 columns: 2 x 6 accumulators
  of w columns in 512), i.e. how many passes of 2 x nacc accumulators cover the product.

``tune`` times every candidate on a seeded synthetic model of that Ndim through
the public call (``Model.surface_spectrum``, host buffers in and out), checks that
every candidate returns the same dos_l / dos_r / dos_bulk (each output element is
summed in the same order whatever the shape; only the convergence norm's block sum
changes order, so they agree to 1e-12 -- a larger difference is a kernel error and
stops the tuner), and keeps the fastest.  Results are stored in a JSON
table keyed by the device (name, SM count, compute capability); ``install`` puts
the entries that match the current device into the library.  The package
installs ``tiles.json`` (next to this file) when the library is first loaded.

Command line (on a GPU):  python -m wannier_tools_gb300.autotune --ndim 40 112 264
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

TABLE = Path(__file__).resolve().with_name("tiles.json")
FORMS = {"fp64": 0, "mixed": 1}
FP64_SMEM_INVERSE_MAX_N = 119   # above this the FP64 kernel's inverse runs in global memory (256 threads)
MIXED_MAX_N = 320


def candidates(form: str, ndim: int) -> list[int]:
    """Launch shapes worth timing at this Ndim ([] = nothing to tune)."""
    if form == "fp64":
        return [128, 256, 512] if 1 <= ndim <= FP64_SMEM_INVERSE_MAX_N else []
    if form == "mixed":
        if not 1 <= ndim <= MIXED_MAX_N:
            return []
        wmax = 40
        npad = (ndim + 7) // 8 * 8
        # passes narrower than 24 columns regenerate the left factor's digits too often;
        # a pass wider than the padded product adds nothing
        return [w for w in range(24, wmax + 1, 8) if w <= npad]
    raise ValueError(f"unknown form {form!r}")


def device_key(info: str) -> str:
    """'NVIDIA GB300, 152 SMs, cc 10.3' from wtg_device_info's string (memory size dropped)."""
    return ", ".join(info.split(", ")[:3])


def shape_for(ndim: int) -> tuple[int, int]:
    """(Num_wann, Np) of the synthetic model used for an Ndim."""
    for np_ in (2, 3, 1):
        if ndim % np_ == 0 and ndim // np_ >= 2:
            return ndim // np_, np_
    return ndim, 1


def default_solves(nsm: int, ndim: int) -> int:
    """Solves per timed call: many waves at small Ndim, where several CTAs share an
    SM and a two-wave sample hides the occupancy a shape gives (about the work of
    two waves at Ndim 112, at least 2 per SM, at most 16384)."""
    return int(min(16384, max(2 * nsm, round(2 * nsm * (112.0 / ndim) ** 3))))


def _time_candidate(api, model, form, ndim, value, kpts, omegas, eta, top, bot, reps):
    prec = FORMS[form]
    before = api.get_tile(prec, ndim)[0]
    api.set_tile(prec, ndim, value)
    try:
        r = model.surface_spectrum(kpts, omegas, eta, top, bot, precision=prec)   # warm-up
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            r = model.surface_spectrum(kpts, omegas, eta, top, bot, precision=prec)
            best = min(best, time.perf_counter() - t0)
    finally:
        api.set_tile(prec, ndim, before)
    return best, r


def tune(ndims, forms=("fp64", "mixed"), reps: int = 3, solves: int | None = None,
         seed: int = 2031, log=print) -> dict:
    """Tile entries {form: {ndim: value}} and their timings for the current device."""
    from . import api, synthetic
    from ._lib import load
    load()
    nsm = int(device_key(api.device_info()).split(", ")[1].split()[0])
    entries: dict = {f: {} for f in forms}
    timings: dict = {f: {} for f in forms}
    for ndim in ndims:
        nsolves = solves or default_solves(nsm, ndim)
        nw, np_ = shape_for(ndim)
        sm = synthetic.make_model(nw, np_, seed=seed + ndim)
        kpts = synthetic.random_kpoints(2, seed=seed)
        omegas = np.linspace(-0.5, 0.5, max(1, nsolves // 2)) / 27.211385
        eta = 1e-3 / 27.211385
        top = list(range(1, nw + 1))
        bot = list(range(1, nw + 1))
        with api.Model.from_surface_model(sm) as model:
            for form in forms:
                cand = candidates(form, ndim)
                if len(cand) < 2:
                    continue
                ref = None
                times = {}
                for v in cand:
                    t, r = _time_candidate(api, model, form, ndim, v, kpts, omegas, eta, top, bot, reps)
                    if ref is None:
                        ref = r
                    else:
                        for name in ("dos_l", "dos_r", "dos_bulk"):
                            if not np.all(np.abs(r[name] - ref[name]) <= 1e-12 * np.abs(ref[name])):
                                raise RuntimeError(f"{form} Ndim {ndim}: tile {v} changed {name}")
                    times[v] = t
                best = min(times, key=times.get)
                entries[form][str(ndim)] = int(best)
                timings[form][str(ndim)] = {str(v): round(t * 1e3, 3) for v, t in times.items()}
                log(f"{form} Ndim {ndim}: " + ", ".join(f"{v}: {t * 1e3:.2f} ms" for v, t in times.items())
                    + f" -> {best}")
    return {"entries": entries, "ms": timings, "reps": reps}


def save(result: dict, device: str, path: Path = TABLE) -> None:
    """Merge one device's entries into the JSON table."""
    table = json.loads(path.read_text()) if path.exists() else {"format": 1, "devices": {}}
    dev = table["devices"].setdefault(device, {"fp64": {}, "mixed": {}})
    for form, ent in result["entries"].items():
        dev.setdefault(form, {}).update(ent)
    dev.setdefault("ms", {})
    for form, ms in result["ms"].items():
        dev["ms"].setdefault(form, {}).update(ms)
    path.write_text(json.dumps(table, indent=1, sort_keys=True) + "\n")


def entries_for(table: dict, device: str) -> dict:
    """{form: {ndim: value}} of one device ({} when the table has none)."""
    dev = table.get("devices", {}).get(device)
    if not dev:
        return {}
    return {f: {int(n): int(v) for n, v in dev.get(f, {}).items()} for f in FORMS}


def install(path: Path = TABLE, device: str | None = None) -> int:
    """Put the table's entries for this device into the library; returns how many."""
    from . import api
    if not path.exists():
        return 0
    table = json.loads(path.read_text())
    dev = device or device_key(api.device_info())
    n = 0
    for form, ent in entries_for(table, dev).items():
        for ndim, v in ent.items():
            api.set_tile(FORMS[form], ndim, v)
            n += 1
    return n


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ndim", type=int, nargs="+", required=True)
    ap.add_argument("--forms", nargs="+", default=["fp64", "mixed"], choices=sorted(FORMS))
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", type=Path, default=TABLE)
    args = ap.parse_args(argv)
    from . import api
    from ._lib import load
    load()
    res = tune(args.ndim, args.forms, reps=args.reps)
    save(res, device_key(api.device_info()), args.out)
    print(json.dumps(res["entries"]))


if __name__ == "__main__":
    main()
