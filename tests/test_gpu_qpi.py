"""Joint density of states / QPI on the GPU against the oracle's sequential
sums (the kernels keep the reference's summation order with unfused
multiply and add, so the results must agree exactly), on spectra computed
by this library."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, synthetic
from wannier_tools_gb300._lib import WtgError

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE


@pytest.mark.parametrize("nk,nom", [(1, 1), (2, 3), (21, 4), (40, 2)])
def test_jdos_kpath_equals_oracle(built_lib, nk, nom):
    rng = np.random.default_rng(nk)
    dos = rng.uniform(0.0, 5.0, (nk, nom))
    assert np.array_equal(api.jdos_kpath(dos), O.jdos_kpath(dos))


def test_jdos_kpath_on_surfstat_spectrum(built_lib):
    m = synthetic.make_model(6, 2, seed=31)
    k = api.kpath_slab([((-0.5, 0.0), (0.5, 0.0))], 25)
    om = np.linspace(-0.5, 0.5, 3) * EV
    with api.Model.from_surface_model(m) as g:
        r = g.surface_spectrum(k, om, 1e-2 * EV, [1, 2], [3, 4])
    _, _, _, l_only, _ = O.surfstat_post(r["dos_l"], r["dos_r"], r["dos_bulk"])
    for d in (r["dos_l"], l_only):
        assert np.array_equal(api.jdos_kpath(d), O.jdos_kpath(d))


@pytest.mark.parametrize("nkx,nky", [(5, 5), (9, 7), (3, 1)])
def test_qpi_kplane_equals_oracle(built_lib, nkx, nky):
    rng = np.random.default_rng(nkx * 10 + nky)
    d = rng.uniform(0.0, 2.0, (nkx, nky))
    p1, p2 = max(1, nkx - 1), max(1, nky - 1)
    got = api.qpi_kplane(d, p1, p2)
    ref = O.qpi_kplane([d], p1, p2, 1.0 / (nkx * nky))
    assert np.array_equal(got, ref)
    # the spin form: four channels, periods from Nk1, Nk2 (here one smaller than nkx, nky)
    ch = [rng.normal(size=(nkx, nky)) for _ in range(4)]
    q1, q2 = max(1, nkx - 2), max(1, nky - 2)
    assert np.array_equal(api.qpi_kplane(ch, q1, q2, 1.0), O.qpi_kplane(ch, q1, q2, 1.0))


def test_qpi_on_arc_plane(built_lib):
    """QPI of an arc computed by the library (11 x 11 plane), through arc_post."""
    m = synthetic.make_model(6, 2, seed=32)
    nkx, nky, k12 = api.kplane_slab(11, 11, (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    with api.Model.from_surface_model(m) as g:
        r = g.surface_spectrum(k12, [0.0], 1e-2 * EV, [1, 2], [3, 4], divide_by_pi=True)
    dl = r["dos_l"][:, 0].reshape(nkx, nky)               # ikp order: j fastest
    l_only, _ = O.arc_post(dl, dl)
    got = api.qpi_kplane(l_only)
    assert np.array_equal(got, O.qpi_kplane([l_only], nkx - 1, nky - 1, 1.0 / (nkx * nky)))


def test_qpi_bad_periods(built_lib):
    with pytest.raises(WtgError):
        api.qpi_kplane(np.ones((3, 3)), 0, 2)
    with pytest.raises(WtgError):
        api.qpi_kplane(np.ones((3, 3)), 4, 2)
