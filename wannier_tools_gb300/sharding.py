"""Multi-process sharding of a surface spectrum over k points.

The reference distributes k round-robin over MPI ranks
(``do ikp = 1+cpuid, knv2, num_cpu``, src/surfstat.f90:123,
src/fermiarc.f90:206) and combines the disjoint rows with SUM reductions of
zero-padded arrays (src/surfstat.f90:201-230, src/fermiarc.f90:336-357).
Every (k, omega) solve is independent, so here each process (one per GPU)
takes a contiguous block of k points -- which keeps each k's Fourier sum on
one device -- and the blocks are gathered on the host.  A gather of disjoint
rows equals the reference's SUM of zero-padded rows.  No device collective is
involved.
"""
from __future__ import annotations

import numpy as np


def block_range(nk: int, world: int, rank: int) -> tuple[int, int]:
    """[start, stop) of rank's contiguous block of nk k points."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    base, extra = divmod(nk, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def roundrobin_indices(nk: int, world: int, rank: int) -> np.ndarray:
    """The reference's k striding: 0-based ikp = rank, rank+world, ..."""
    return np.arange(rank, nk, world)


def spectrum_sharded(compute, kpts, omegas, group=None, keys=("dos_l", "dos_r", "dos_bulk", "iters", "status")):
    """Run ``compute(k_block, omegas) -> dict of (nk_block, nomega) arrays`` on
    this rank's block and gather the full (nk, nomega) arrays on every rank
    (torch.distributed, any backend; a single process needs no group)."""
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 2)
    nk = kpts.shape[0]
    try:
        import torch.distributed as dist
        active = dist.is_available() and dist.is_initialized()
    except Exception:
        active = False
    world = dist.get_world_size(group) if active else 1
    rank = dist.get_rank(group) if active else 0
    s, e = block_range(nk, world, rank)
    local = compute(kpts[s:e], omegas) if e > s else None
    parts = [None] * world
    if active:
        dist.all_gather_object(parts, (s, e, None if local is None else {k: local[k] for k in keys}), group=group)
    else:
        parts = [(s, e, None if local is None else {k: local[k] for k in keys})]
    nwo = len(np.asarray(omegas).ravel())
    out = {}
    for name in keys:
        ref = next((p[2][name] for p in parts if p[2] is not None), None)
        dtype = ref.dtype if ref is not None else np.float64
        full = np.zeros((nk, nwo), dtype=dtype)
        for ps, pe, d in parts:
            if d is not None:
                full[ps:pe] = d[name]
        out[name] = full
    return out
