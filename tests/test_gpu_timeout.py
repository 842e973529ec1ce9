"""Bounded waits of the mixed (tensor-core) kernels run out cleanly on the GPU.

Every mbarrier wait of the split-BF16 pipeline has an iteration limit; when it
runs out the CTA stops issuing MMAs, the point gets WTG_PT_TIMEOUT, the CTA
waits (with the built-in bound) for the MMAs it already committed, frees its
tensor memory and returns, and the host call returns normally.  The test-only
switch WTG_TEST_MIXED_SPIN_LIMIT shortens the pipeline waits to one
non-blocking poll, which runs out while the tensor cores are still busy: a
wait that no MMA completion can satisfy in time, not a fault.  Afterwards the
same context computes the same spectra as before, bit for bit."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import _lib, api, synthetic
from wannier_tools_gb300._lib import PREC_MIXED, PT_TIMEOUT

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE


def _with_spin_limit(lib, n, fn):
    assert lib.wtg_test_option(_lib.TEST_MIXED_SPIN_LIMIT, n) == _lib.WTG_OK
    try:
        return fn()
    finally:
        assert lib.wtg_test_option(_lib.TEST_MIXED_SPIN_LIMIT, 0) == _lib.WTG_OK


@pytest.mark.parametrize("nw,np_", [(20, 2), (56, 2)])
def test_mixed_pipeline_waits_run_out(built_lib, nw, np_):
    m = synthetic.make_model(nw, np_, seed=900 + nw)
    kp = synthetic.random_kpoints(4, seed=nw)
    om = np.array([-0.2, 0.1, 0.3]) * EV
    top, bot = list(range(1, nw + 1, 2)), list(range(1, nw + 1, 3))
    with api.Model.from_surface_model(m) as g:
        before = g.surface_spectrum(kp, om, 1e-2 * EV, top, bot, precision=PREC_MIXED)
        assert (before["status"] == 0).all()
        timed = _with_spin_limit(built_lib, 1, lambda: g.surface_spectrum(
            kp, om, 1e-2 * EV, top, bot, precision=PREC_MIXED))
        # every point flagged, the call itself returned normally
        assert ((timed["status"] & PT_TIMEOUT) != 0).all(), timed["status"]
        after = g.surface_spectrum(kp, om, 1e-2 * EV, top, bot, precision=PREC_MIXED)
    for name in ("dos_l", "dos_r", "dos_bulk", "iters", "status"):
        assert np.array_equal(after[name], before[name]), name


def test_batch_mixed_waits_run_out(built_lib):
    """The uneven-batch kernel: points pulled after a CTA gave up are marked too."""
    shapes = [(8, 2), (20, 2)]
    ms = [synthetic.make_model(nw, np_, seed=950 + i) for i, (nw, np_) in enumerate(shapes)]
    gs = [api.Model.from_surface_model(m) for m in ms]
    try:
        tops = [list(range(1, m.nw + 1)) for m in ms]
        rng = np.random.default_rng(4)
        n = 400                                    # more points than CTAs: some CTAs pull again
        pm = rng.integers(0, 2, n).astype(np.int32)
        k = rng.uniform(-0.5, 0.5, (n, 2))
        om = rng.uniform(-1, 1, n) * EV
        eta = np.full(n, 1e-2 * EV)
        timed = _with_spin_limit(built_lib, 1, lambda: api.batch_spectrum(
            gs, tops, tops, pm, k, om, eta, precision=PREC_MIXED))
        assert ((timed["status"] & PT_TIMEOUT) != 0).all()
        after = api.batch_spectrum(gs, tops, tops, pm, k, om, eta, precision=PREC_MIXED)
        assert (after["status"] == 0).all()
        assert np.isfinite(after["dos_l"]).all()
    finally:
        for g in gs:
            g.close()
