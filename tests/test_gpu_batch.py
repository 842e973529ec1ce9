"""Uneven batches (several models of different Ndim, eta per point) in one
persistent launch, and the request loop on the GPU.

Each point of a batch runs the same per-point arithmetic as the per-model
path (Fourier sum in the same order, the same decimation), so the batch must
match wtg_surface_spectrum point for point to 1e-12 (the norm test's block
sum is the only reduction whose order may differ) and the oracle to 1e-9
(FP64) / 1e-5 (mixed).  A request's result through the serving loop must be
bit-identical alone and in a mix."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, synthetic
from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED, WtgError

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE
SHAPES = [(8, 2), (20, 2), (13, 3), (44, 3)]        # Ndim 16, 40, 39, 132


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.fixture(scope="module")
def models(built_lib):
    ms = [synthetic.make_model(nw, np_, seed=500 + i) for i, (nw, np_) in enumerate(SHAPES)]
    gs = [api.Model.from_surface_model(m) for m in ms]
    yield ms, gs
    for g in gs:
        g.close()


def _points(n, nmodels, seed):
    rng = np.random.default_rng(seed)
    pm = rng.integers(0, nmodels, n).astype(np.int32)
    k = rng.uniform(-0.5, 0.5, (n, 2))
    om = rng.uniform(-1, 1, n) * EV
    eta = np.exp(rng.uniform(np.log(1e-3), np.log(1e-2), n)) * EV
    return pm, k, om, eta


def _lists(ms):
    tops = [list(range(1, m.nw + 1, 2)) for m in ms]
    bots = [list(range(1, m.nw + 1, 3)) for m in ms]
    return tops, bots


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_batch_matches_per_model_path(models, prec):
    ms, gs = models
    tops, bots = _lists(ms)
    pm, k, om, eta = _points(24, len(ms), seed=1 + prec)
    got = api.batch_spectrum(gs, tops, bots, pm, k, om, eta, precision=prec)
    for p in range(len(pm)):
        g = gs[pm[p]]
        ref = g.surface_spectrum(k[p:p + 1], om[p:p + 1], eta[p], tops[pm[p]], bots[pm[p]], precision=prec)
        for name in ("dos_l", "dos_r", "dos_bulk"):
            assert rel(got[name][p], ref[name][0, 0]) <= 1e-12, (p, name)
        assert abs(int(got["iters"][p]) - int(ref["iters"][0, 0])) <= 1
    assert (got["status"] == 0).all()


def test_batch_fp64_vs_oracle(models):
    ms, gs = models
    tops, bots = _lists(ms)
    pm, k, om, eta = _points(8, len(ms), seed=7)
    got = api.batch_spectrum(gs, tops, bots, pm, k, om, eta, precision=PREC_FP64)
    for p in range(len(pm)):
        m = ms[pm[p]]
        ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, k[p:p + 1], om[p:p + 1],
                                 eta[p], tops[pm[p]], bots[pm[p]])
        for name in ("dos_l", "dos_r", "dos_bulk"):
            assert rel(got[name][p], ref[name][0, 0]) <= 1e-9, (p, name)


def test_engine_reuse_and_errors(models):
    ms, gs = models
    tops, bots = _lists(ms)
    pm, k, om, eta = _points(10, len(ms), seed=3)
    with api.Engine(gs, tops, bots, precision=PREC_FP64, max_points=16) as e:
        a = e.run(pm, k, om, eta)
        b = e.run(pm, k, om, eta)
        for name in ("dos_l", "dos_r", "dos_bulk", "iters"):
            assert np.array_equal(a[name], b[name])
        info = e.info()
        assert info["launches"] == 2 and info["device_bytes"] > 0
        with pytest.raises(WtgError):
            e.run(np.full(3, 9, np.int32), k[:3], om[:3], eta[:3])      # no model 9
        with pytest.raises(WtgError):
            e.run(np.zeros(17, np.int32), np.zeros((17, 2)), np.zeros(17), np.full(17, 1e-4))
        # order inside a batch does not matter
        perm = np.random.default_rng(0).permutation(len(pm))
        c = e.run(pm[perm], k[perm], om[perm], eta[perm])
        for name in ("dos_l", "dos_r", "dos_bulk"):
            assert np.array_equal(c[name], a[name][perm])


def test_large_ndim_in_uneven_batch(built_lib):
    """Ndim 16 and 264 points interleaved in one FP64 launch (global-memory
    inverse for the large model, shared-memory inverse for the small one)."""
    ms = [synthetic.make_model(8, 2, seed=1), synthetic.make_model(88, 3, seed=2)]
    gs = [api.Model.from_surface_model(m) for m in ms]
    try:
        tops, bots = [[1, 2], [1, 5]], [[3], [7, 8]]
        pm = np.array([1, 0, 0, 1, 0], np.int32)
        rng = np.random.default_rng(4)
        k = rng.uniform(-0.5, 0.5, (5, 2))
        om = rng.uniform(-0.5, 0.5, 5) * EV
        eta = np.full(5, 1e-2 * EV)
        got = api.batch_spectrum(gs, tops, bots, pm, k, om, eta, precision=PREC_FP64)
        for p in (0, 1):
            m = ms[pm[p]]
            ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, k[p:p + 1], om[p:p + 1],
                                     eta[p], tops[pm[p]], bots[pm[p]])
            for name in ("dos_l", "dos_r", "dos_bulk"):
                assert rel(got[name][p], ref[name][0, 0]) <= 1e-9
    finally:
        for g in gs:
            g.close()


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_serving_alone_equals_in_mix(models, prec):
    from wannier_tools_gb300.serving import SurfaceServer
    ms, gs = models
    tops, bots = _lists(ms)
    rng = np.random.default_rng(11)
    reqs = []
    for i in range(12):
        n = int(rng.integers(10, 60))
        reqs.append((int(rng.integers(len(ms))), rng.uniform(-0.5, 0.5, (1, 2)),
                     np.linspace(*np.sort(rng.uniform(-1, 1, 2)), n) * EV,
                     float(rng.uniform(1e-3, 1e-2)) * EV))
    with SurfaceServer(gs, tops, bots, precision=prec, slot_points=128, max_slots=3) as srv:
        alone = srv.submit(*reqs[5]).result(timeout=600)
        futs = [srv.submit(*r) for r in reqs]                  # all at once: batched and overlapped
        mixed = [f.result(timeout=600) for f in futs]
        assert len(srv.batches) >= 2
    for name in ("dos_l", "dos_r", "dos_bulk", "iters", "status"):
        assert np.array_equal(alone[name], mixed[5][name]), name
    ref = gs[reqs[5][0]].surface_spectrum(reqs[5][1], reqs[5][2], reqs[5][3], tops[reqs[5][0]],
                                          bots[reqs[5][0]], precision=prec)
    assert rel(alone["dos_bulk"], ref["dos_bulk"][0]) <= 1e-12


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_serving_model_added_while_running(models, prec):
    """A model registered while requests are in flight is served by an engine built
    after it, with the per-model path's result (1e-12; the same per-point arithmetic)."""
    from wannier_tools_gb300.serving import SurfaceServer
    ms, gs = models
    tops, bots = _lists(ms)
    extra = synthetic.make_model(30, 2, seed=777)                  # Ndim 60
    with api.Model.from_surface_model(extra) as g_extra:
        with SurfaceServer(gs[:2], tops[:2], bots[:2], precision=prec, slot_points=128,
                           max_slots=2) as srv:
            busy = [srv.submit(i % 2, [[0.1 * i, 0.2]], np.linspace(-0.5, 0.5, 60) * EV, 5e-3 * EV)
                    for i in range(4)]
            mid = srv.add_model(g_extra, list(range(1, 31, 2)), list(range(1, 31, 3)))
            om = np.linspace(-0.3, 0.4, 50) * EV
            got = srv.submit(mid, [[0.25, -0.1]], om, 4e-3 * EV).result(timeout=600)
            for f in busy:
                assert (f.result(timeout=600)["status"] == 0).all()
            assert srv.engines_built >= 2
        ref = g_extra.surface_spectrum([[0.25, -0.1]], om, 4e-3 * EV, list(range(1, 31, 2)),
                                       list(range(1, 31, 3)), precision=prec)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert rel(got[name], ref[name][0]) <= 1e-12, name
