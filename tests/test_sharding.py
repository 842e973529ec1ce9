"""Multi-process path on CPU: world_size-2 gloo ranks shard k points and the
gathered spectrum equals the unsharded one (the oracle stands in for the GPU
compute so the sharding logic itself is what is tested)."""
import os
import socket

import numpy as np
import pytest

from wannier_tools_gb300 import sharding

EV = 1.0 / 27.211385


def test_block_range_covers_disjointly():
    for nk in (0, 1, 5, 40401):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                s, e = sharding.block_range(nk, world, r)
                seen.extend(range(s, e))
            assert seen == list(range(nk))
    with pytest.raises(ValueError):
        sharding.block_range(4, 2, 2)


def test_roundrobin_matches_reference_striding():
    # do ikp = 1+cpuid, knv2, num_cpu  (1-based) -> 0-based rank, rank+world, ...
    got = sharding.roundrobin_indices(10, 3, 1)
    assert list(got) == [1, 4, 7]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    import torch.distributed as dist

    from oracle import wt_oracle as O
    from wannier_tools_gb300 import sharding as S
    from wannier_tools_gb300 import synthetic
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    m = synthetic.make_model(3, 2, seed=21)
    kp = synthetic.random_kpoints(5, seed=2)
    om = np.array([-0.2, 0.3]) * EV

    def compute(kb, omegas):
        return O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, 3, 2, kb, omegas, 1e-2 * EV, [1, 2], [3])

    out = S.spectrum_sharded(compute, kp, om)
    if rank == 0:
        q.put({k: v for k, v in out.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_gather_equals_unsharded():
    import multiprocessing as mp

    from oracle import wt_oracle as O
    from wannier_tools_gb300 import synthetic
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    m = synthetic.make_model(3, 2, seed=21)
    kp = synthetic.random_kpoints(5, seed=2)
    om = np.array([-0.2, 0.3]) * EV
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, 3, 2, kp, om, 1e-2 * EV, [1, 2], [3])
    for name in ("dos_l", "dos_r", "dos_bulk", "iters"):
        assert np.array_equal(got[name], ref[name])
