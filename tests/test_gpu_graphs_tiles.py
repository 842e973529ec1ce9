"""CUDA-graph replays of engine runs and the autotuner's tile table, on the GPU.

A run replayed from a captured graph stages the same points (the count and the
run's scalars in a device header) and launches the same kernel, so its results
must be bit-identical to a direct launch for any point count.  A tile (FP64
threads per CTA, mixed pass width) changes how output elements are spread over
threads and passes, never the order in which one element is summed; only the
convergence norm's block sum is taken in another order, so spectra agree to
1e-12 and iteration counts to one step."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, autotune, synthetic
from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE
SHAPES = [(8, 2), (20, 2), (56, 2)]        # Ndim 16, 40, 112


@pytest.fixture(scope="module")
def models(built_lib):
    ms = [synthetic.make_model(nw, np_, seed=700 + i) for i, (nw, np_) in enumerate(SHAPES)]
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


def _same(a, b):
    for name in ("dos_l", "dos_r", "dos_bulk", "iters", "status"):
        assert np.array_equal(a[name], b[name]), name


def _close(a, b):
    for name in ("dos_l", "dos_r", "dos_bulk"):
        x, y = np.asarray(a[name]), np.asarray(b[name])
        assert np.all(np.abs(x - y) <= 1e-12 * np.abs(y)), name
    assert np.max(np.abs(a["iters"].astype(int) - b["iters"].astype(int))) <= 1
    assert np.array_equal(a["status"], b["status"])


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_graph_replays_match_direct_launches(models, prec):
    ms, gs = models
    tops = [list(range(1, m.nw + 1)) for m in ms]
    bots = [list(range(1, m.nw + 1, 2)) for m in ms]
    with api.Engine(gs, tops, bots, precision=prec, max_points=300, graphs=True) as eg, \
            api.Engine(gs, tops, bots, precision=prec, max_points=300, graphs=False) as ed:
        for i, n in enumerate((1, 5, 64, 65, 300, 40, 65)):
            pm, k, om, eta = _points(n, len(gs), seed=10 * prec + i)
            tol, itermax, dbp = (1e-10, 60, i % 2 == 0) if i % 3 else (O.ACCURACY_REF, 100, False)
            a = eg.run(pm, k, om, eta, tol=tol, itermax=itermax, divide_by_pi=dbp)
            b = ed.run(pm, k, om, eta, tol=tol, itermax=itermax, divide_by_pi=dbp)
            _same(a, b)
        gi = eg.graph_info()
        # capacities 64 (n = 1, 5, 64, 40), 128 (n = 65, twice), 300 (the engine's max_points)
        assert gi == {"graphs": 3, "graph_launches": 7}
        assert ed.graph_info() == {"graphs": 0, "graph_launches": 0}
        assert eg.info()["launches"] == 7


def test_graph_replay_matches_the_per_model_call(models):
    """A graph-replayed batch point equals the per-model call (1e-12, as the
    batch tests' bound) for the largest model."""
    ms, gs = models
    top, bot = list(range(1, ms[2].nw + 1)), list(range(1, ms[2].nw + 1))
    with api.Engine([gs[2]], [top], [bot], precision=PREC_MIXED, max_points=64) as e:
        pm = np.zeros(3, np.int32)
        k = np.array([[0.1, 0.2], [-0.3, 0.4], [0.0, 0.0]])
        om = np.array([0.0, 0.1, -0.2]) * EV
        eta = np.full(3, 1e-3 * EV)
        got = e.run(pm, k, om, eta)
        for p in range(3):
            ref = gs[2].surface_spectrum(k[p:p + 1], om[p:p + 1], eta[p], top, bot, precision=PREC_MIXED)
            for name in ("dos_l", "dos_r", "dos_bulk"):
                r = float(ref[name].ravel()[0])
                assert abs(got[name][p] - r) <= 1e-12 * abs(r), name


@pytest.mark.parametrize("form,ndim_model", [("fp64", 1), ("fp64", 2), ("mixed", 2), ("mixed", 1)])
def test_every_tile_gives_the_same_spectrum(models, form, ndim_model):
    ms, gs = models
    m, g = ms[ndim_model], gs[ndim_model]
    ndim = m.nw * m.np_
    prec = autotune.FORMS[form]
    cands = autotune.candidates(form, ndim)
    assert len(cands) >= 2
    k = synthetic.random_kpoints(3, seed=5)
    om = np.linspace(-0.3, 0.3, 4) * EV
    top, bot = list(range(1, m.nw + 1)), list(range(1, m.nw + 1, 3))
    before = api.get_tile(prec, ndim)[0]
    try:
        ref = None
        for v in cands:
            api.set_tile(prec, ndim, v)
            assert api.get_tile(prec, ndim)[0] == v
            r = g.surface_spectrum(k, om, 2e-3 * EV, top, bot, precision=prec)
            if ref is None:
                ref = r
            else:
                _close(r, ref)
    finally:
        api.set_tile(prec, ndim, before)


def test_mixed_engine_with_tuned_widths(models):
    """Engines take the pass widths in force when they are created; widths
    other than the built-in ones (40 columns at both Ndim) give the same batch."""
    ms, gs = models
    tops = [list(range(1, m.nw + 1)) for m in ms]
    bots = [list(range(1, m.nw + 1, 2)) for m in ms]
    pm, k, om, eta = _points(40, len(gs), seed=99)
    with api.Engine(gs, tops, bots, precision=PREC_MIXED, max_points=64) as e:
        ref = e.run(pm, k, om, eta)
    saved = {m.nw * m.np_: api.get_tile(PREC_MIXED, m.nw * m.np_)[0] for m in ms}
    try:
        api.set_tile(PREC_MIXED, 40, 24)
        api.set_tile(PREC_MIXED, 112, 32)
        with api.Engine(gs, tops, bots, precision=PREC_MIXED, max_points=64) as e:
            got = e.run(pm, k, om, eta)
        _close(got, ref)
    finally:
        for n, v in saved.items():
            api.set_tile(PREC_MIXED, n, v)


def test_tuner_picks_a_candidate(built_lib, tmp_path):
    res = autotune.tune([40], forms=("fp64", "mixed"), reps=1, solves=64, log=lambda *_: None)
    assert res["entries"]["fp64"]["40"] in autotune.candidates("fp64", 40)
    assert res["entries"]["mixed"]["40"] in autotune.candidates("mixed", 40)
    dev = autotune.device_key(api.device_info())
    autotune.save(res, dev, tmp_path / "t.json")
    n = autotune.install(tmp_path / "t.json")
    assert n == 2
    autotune.install()          # the package table again
