"""Phonon forms: the LO-TO corrected principal-layer Hamiltonian
(ham_qlayer2qlayer_LOTO) and the squared energies of the drivers, on the GPU
against the oracle (Fourier sums to 1e-12 relative to the largest entry,
spectra at the plain form's 1e-9)."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, synthetic
from wannier_tools_gb300._lib import WtgError

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE


def phonon_model(natoms, np_, seed):
    m = synthetic.make_model(3 * natoms, np_, seed=seed)
    rng = np.random.default_rng(seed)
    born = rng.normal(scale=1.0, size=(natoms, 3, 3))
    a = rng.normal(size=(3, 3))
    diele = a @ a.T + 3.0 * np.eye(3)                      # positive definite
    masses = rng.uniform(10.0, 100.0, natoms)
    return m, (born, diele, masses, 150.0)


@pytest.mark.parametrize("k", [(0.13, -0.27), (0.0, 0.0), (0.005, -0.004), (0.5, 0.5)])
def test_loto_fourier_sum(built_lib, k):
    m, loto = phonon_model(2, 2, seed=71)
    with api.Model.from_surface_model(m) as g:
        g.set_loto(*loto)
        a00, a01 = g.ham_qlayer2qlayer(k)
        g.set_loto(None)
        p00, _ = g.ham_qlayer2qlayer(k)
    b00, b01 = O.ham_qlayer2qlayer_loto(k, m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, *loto)
    scale = max(np.abs(b00).max(), np.abs(b01).max())
    assert np.abs(a00 - b00).max() <= 1e-12 * scale
    assert np.abs(a01 - b01).max() <= 1e-12 * scale
    assert np.abs(a00 - p00).max() > 1e-6 * scale          # the correction is really applied


def test_loto_arc_spectrum(built_lib):
    m, loto = phonon_model(2, 2, seed=72)
    kp = np.array([[0.1, 0.2], [0.003, 0.002], [-0.3, 0.4]])
    om = np.array([0.05]) ** 2                             # phonon: energy squared
    with api.Model.from_surface_model(m) as g:
        g.set_loto(*loto)
        got = g.surface_spectrum(kp, om, 1e-3, [1, 2], [3, 4], divide_by_pi=True)
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, kp, om, 1e-3, [1, 2], [3, 4],
                             scale=1.0 / O.PI_REF, loto=loto)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert np.max(np.abs(got[name] - ref[name]) / np.abs(ref[name])) <= 1e-9, name


def test_phonon_drivers_square_energies(built_lib):
    m = synthetic.make_model(3, 2, seed=73)
    with api.Model.from_surface_model(m) as g:
        e = api.surfstat(g, api.kpath_slab([((0.0, 0.0), (0.5, 0.0))], 4), 0.1, 0.3, 4, [1], [1])
        p = api.surfstat(g, api.kpath_slab([((0.0, 0.0), (0.5, 0.0))], 4), 0.1, 0.3, 4, [1], [1],
                         particle="phonon")
        assert np.allclose(p["omega"], e["omega"] ** 2) and p["eta"] == e["eta"]
        direct = g.surface_spectrum(api.kpath_slab([((0.0, 0.0), (0.5, 0.0))], 4), e["omega"] ** 2,
                                    e["eta"], [1], [1])
        assert np.array_equal(p["dos_l"], direct["dos_l"])


def test_loto_argument_checks(built_lib):
    m = synthetic.make_model(4, 1, seed=74)                 # Num_wann 4: not 3 x natoms
    with api.Model.from_surface_model(m) as g:
        with pytest.raises(WtgError):
            g.set_loto(np.ones((1, 3, 3)), np.eye(3), [1.0], 10.0)
    m, loto = phonon_model(1, 1, seed=75)
    with api.Model.from_surface_model(m) as g:
        g.set_loto(*loto)
        with pytest.raises(WtgError):                       # engines take plain models only
            api.Engine([g], [[1]], [[1]])
