"""FP64 decimation at large Ndim (above 119, up to 320), where the inverse runs
in global memory in panels of pivot steps.

The panel variant applies the same operations in the same order as the
shared-memory Gauss-Jordan, so at Ndim <= 119, forced onto the panel variant,
it must reproduce the shared-memory kernel bit for bit; above 119 it is checked
against the oracle at the 1e-9 relative bound of the plain form."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import _lib, api, synthetic
from wannier_tools_gb300._lib import PREC_FP64

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE
RTOL = 1e-9


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b) / np.maximum(np.abs(b), 1e-300)))


def nrel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _spectrum(m, kp, om, eta, top, bot, spin=False, force_global=False):
    # the test-only switch that makes the FP64 kernel invert in global memory at any Ndim
    lib = _lib.load()
    assert lib.wtg_test_option(_lib.TEST_FP64_GLOBAL_INVERSE, 1 if force_global else 0) == 0
    try:
        with api.Model.from_surface_model(m) as g:
            if spin:
                return g.surface_spectrum_spin(kp, om, eta, top, bot, arc=True)
            return g.surface_spectrum(kp, om, eta, top, bot)
    finally:
        lib.wtg_test_option(_lib.TEST_FP64_GLOBAL_INVERSE, 0)


@pytest.mark.parametrize("nw,np_", [(3, 1), (20, 2), (13, 3), (56, 2)])
def test_panel_inverse_bitwise_equals_shared_memory(built_lib, nw, np_):
    m = synthetic.make_model(nw, np_, seed=40 + nw)
    kp = synthetic.random_kpoints(5, seed=nw)
    om = np.array([-0.3, 0.0, 0.2]) * EV
    top, bot = [1, 2, 3][:nw], [1, nw]
    a = _spectrum(m, kp, om, 1e-3 * EV, top, bot)
    b = _spectrum(m, kp, om, 1e-3 * EV, top, bot, force_global=True)
    for name in ("dos_l", "dos_r", "dos_bulk", "iters", "status"):
        assert np.array_equal(a[name], b[name]), name


def test_panel_inverse_bitwise_spin(built_lib):
    m = synthetic.make_model(8, 2, seed=77)
    kp = synthetic.random_kpoints(3, seed=5)
    om = np.array([0.1]) * EV
    a = _spectrum(m, kp, om, 1e-2 * EV, [1, 2, 5], [1, 4], spin=True)
    b = _spectrum(m, kp, om, 1e-2 * EV, [1, 2, 5], [1, 4], spin=True, force_global=True)
    for name in ("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r", "dos_l"):
        assert np.array_equal(a[name], b[name]), name


@pytest.mark.parametrize("nw,np_,nk", [(44, 3, 3), (64, 2, 2), (88, 3, 2)])
def test_large_ndim_vs_oracle(built_lib, nw, np_, nk):
    """Ndim 132, 128 and 264 (the Num_wann = 88, Np = 3 model) at eta = 1e-3 eV."""
    m = synthetic.make_model(nw, np_, seed=nw + np_)
    kp = synthetic.random_kpoints(nk, seed=nw)
    om = np.array([0.05]) * EV
    top = list(range(1, nw + 1, 2))
    bot = list(range(2, nw + 1, 3))
    got = _spectrum(m, kp, om, 1e-3 * EV, top, bot)
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, kp, om, 1e-3 * EV, top, bot)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        e = rel(got[name], ref[name])
        print("large Ndim", nw * np_, name, e)
        assert e <= RTOL, (name, e)
    assert np.abs(got["iters"] - ref["iters"]).max() <= 1
    assert (got["status"] == 0).all()


@pytest.mark.parametrize("n", [120, 200, 264, 320])
def test_unit_ops_large(built_lib, n):
    rng = np.random.default_rng(n)
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    b = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    assert nrel(api.mat_mul(a, b, PREC_FP64), a @ b) <= 1e-14
    g, st = api.inv(a + 3.0 * np.sqrt(n) * np.eye(n), PREC_FP64)
    assert st == 0 and nrel(g, np.linalg.inv(a + 3.0 * np.sqrt(n) * np.eye(n))) <= 1e-13


def test_surfgreen_1985_large_full_matrices(built_lib):
    nw, np_ = 75, 2
    m = synthetic.make_model(nw, np_, seed=9)
    h00, h01 = O.ham_qlayer2qlayer([0.21, -0.4], m.hmnr, m.irvec, m.ndegen, nw, np_)
    ref = O.surfgreen_1985(0.03 * EV, h00, h01, 1e-2 * EV)
    got = api.surfgreen_1985(0.03 * EV, h00, h01, 1e-2 * EV)
    for a, b in zip(got[:3], ref[:3]):
        assert nrel(a, b) <= RTOL
    assert abs(got[3] - ref[3]) <= 1


def test_singular_pivot_large(built_lib):
    """An exactly singular matrix at Ndim 150: status flags it and the result is
    the identity, as the shared-memory inverse does."""
    n = 150
    a = np.zeros((n, n), complex)
    a[: n - 1, : n - 1] = np.eye(n - 1) * 2.0
    g, st = api.inv(a, PREC_FP64)
    assert st != 0
    assert np.array_equal(g, np.eye(n))
