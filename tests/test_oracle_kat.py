"""Pins the CPU oracle against closed-form known answers (no GPU).

The reference ships no golden outputs for surfgreen_1985, so the oracle's
restatement of src/surfgreen.f90 / src/ham_qlayer2qlayer.f90 is checked
against physics that has an exact answer."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import synthetic

EV = O.EV2HARTREE


def chain_h(np_, e0, t):
    m = synthetic.chain_model(e0, t)
    return O.ham_qlayer2qlayer([0.0, 0.0], m.hmnr, m.irvec, m.ndegen, 1, np_)


@pytest.mark.parametrize("eta_ev", [1e-2, 1e-3])
@pytest.mark.parametrize("w_ev", [-2.5, -1.0, 0.0, 0.3, 1.7, 2.9])
def test_chain_closed_form(w_ev, eta_ev):
    e0, t = 0.3, 1.0
    h00, h01 = chain_h(1, e0, t)
    gll, grr, gb, it, st = O.surfgreen_1985(w_ev * EV, h00, h01, eta_ev * EV)
    gs, gbk = O.chain_surface_gf(complex(w_ev * EV, eta_ev * EV), e0 * EV, t * EV)
    assert st == 0 and 1 <= it < 100
    assert abs(gll[0, 0] - gs) <= 1e-10 * abs(gs)
    assert abs(grr[0, 0] - gs) <= 1e-10 * abs(gs)
    assert abs(gb[0, 0] - gbk) <= 1e-10 * abs(gbk)


def test_chain_two_layer_cell_equals_one_layer():
    e0, t = -0.2, 0.7
    a00, a01 = chain_h(1, e0, t)
    b00, b01 = chain_h(2, e0, t)
    assert np.allclose(b00, [[e0 * EV, t * EV], [t * EV, e0 * EV]])
    assert np.allclose(b01, [[0, 0], [t * EV, 0]])
    for w in (-0.9, 0.1, 1.2):
        g1 = O.surfgreen_1985(w * EV, a00, a01, 5e-3 * EV)
        g2 = O.surfgreen_1985(w * EV, b00, b01, 5e-3 * EV)
        assert abs(g2[0][0, 0] - g1[0][0, 0]) <= 1e-9 * abs(g1[0][0, 0])     # top site
        assert abs(g2[1][1, 1] - g1[1][0, 0]) <= 1e-9 * abs(g1[1][0, 0])     # bottom site
        tr = g2[2][0, 0] + g2[2][1, 1]
        assert abs(tr - 2 * g1[2][0, 0]) <= 1e-9 * abs(g1[2][0, 0])


def test_rotated_decoupled_chains_trace():
    """Unitary-rotated decoupled chains: traces of GLL / GB are invariant."""
    rng = np.random.default_rng(3)
    e0 = np.array([-0.4, 0.1, 0.5])
    t = np.array([0.8, 1.1, 0.6])
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3)))
    h = np.zeros((3, 3, 3), np.complex128)
    h[0] = q @ np.diag(t) @ q.conj().T
    h[1] = q @ np.diag(e0) @ q.conj().T
    h[2] = q @ np.diag(t) @ q.conj().T
    irv = np.array([[0, 0, -1], [0, 0, 0], [0, 0, 1]], np.int32)
    res = O.surface_spectrum(h * EV, irv, np.ones(3, np.int32), 3, 1, [[0.1, 0.2]],
                             np.array([-0.5, 0.05, 0.9]) * EV, 4e-3 * EV, [1, 2, 3], [1, 2, 3])
    for j, w in enumerate([-0.5, 0.05, 0.9]):
        z = complex(w * EV, 4e-3 * EV)
        gs = sum(O.chain_surface_gf(z, a * EV, b * EV)[0] for a, b in zip(e0, t))
        gbk = sum(O.chain_surface_gf(z, a * EV, b * EV)[1] for a, b in zip(e0, t))
        assert abs(res["dos_l"][0, j] + gs.imag) <= 1e-9 * abs(gs)
        assert abs(res["dos_r"][0, j] + gs.imag) <= 1e-9 * abs(gs)
        assert abs(res["dos_bulk"][0, j] + gbk.imag) <= 1e-9 * abs(gbk)


def test_hamiltonian_hermitian_and_bloch():
    """H00 Hermitian; H00 + H01 e^{i th} + H01^dag e^{-i th} at th = 0 has the
    spectrum of H(k1, k2, k3 = n/Np), n = 0..Np-1 (Np-fold supercell)."""
    m = synthetic.make_model(3, 2, seed=5, rmax=1)
    k = np.array([0.13, -0.31])
    h00, h01 = O.ham_qlayer2qlayer(k, m.hmnr, m.irvec, m.ndegen, m.nw, 2)
    assert np.allclose(h00, h00.conj().T, atol=1e-15)
    slab = h00 + h01 + h01.conj().T
    ev_slab = np.sort(np.linalg.eigvalsh(slab))
    ev = []
    for n in range(2):
        k3 = n / 2.0
        hk = sum(m.hmnr[r] * np.exp(2j * np.pi * (k[0] * m.irvec[r, 0] + k[1] * m.irvec[r, 1] + k3 * m.irvec[r, 2]))
                 for r in range(m.nrpts))
        ev.extend(np.linalg.eigvalsh(hk))
    assert np.allclose(ev_slab, np.sort(ev), atol=1e-12)


def test_surface_gf_equals_thick_slab_block():
    """GLL / GRR equal the end blocks of (w - H_slab)^-1 for a thick slab."""
    m = synthetic.make_model(4, 2, seed=9, rmax=1)
    h00, h01 = O.ham_qlayer2qlayer([0.2, -0.1], m.hmnr, m.irvec, m.ndegen, m.nw, 2)
    n = h00.shape[0]
    L = 160
    w = complex(0.1 * EV, 0.2 * EV)
    big = np.zeros((L * n, L * n), np.complex128)
    for i in range(L):
        big[i * n:(i + 1) * n, i * n:(i + 1) * n] = h00
        if i + 1 < L:
            big[i * n:(i + 1) * n, (i + 1) * n:(i + 2) * n] = h01
            big[(i + 1) * n:(i + 2) * n, i * n:(i + 1) * n] = h01.conj().T
    gfull = np.linalg.inv(w * np.eye(L * n) - big)
    gll, grr, gb, it, st = O.surfgreen_1985(w.real, h00, h01, w.imag)
    assert np.allclose(gll, gfull[:n, :n], rtol=0, atol=1e-7 * np.abs(gll).max())
    assert np.allclose(grr, gfull[-n:, -n:], rtol=0, atol=1e-7 * np.abs(grr).max())
    mid = (L // 2) * n
    assert np.allclose(gb, gfull[mid:mid + n, mid:mid + n], rtol=0, atol=1e-7 * np.abs(gb).max())


def test_spectral_positivity():
    m = synthetic.make_model(5, 2, seed=2)
    res = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, 2, [[0.0, 0.0], [0.3, 0.4]],
                             np.linspace(-1, 1, 4) * EV, 1e-2 * EV, list(range(1, 6)), list(range(1, 6)))
    assert (res["dos_l"] > 0).all() and (res["dos_r"] > 0).all() and (res["dos_bulk"] > 0).all()
    assert (res["status"] == 0).all()


def test_itermax_zero_and_not_converged_flag():
    m = synthetic.make_model(2, 1, seed=1)
    h00, h01 = O.ham_qlayer2qlayer([0, 0], m.hmnr, m.irvec, m.ndegen, 2, 1)
    *_, it, st = O.surfgreen_1985(0.0, h00, h01, 1e-4, itermax=0)
    assert it == 0 and st & O.ST_NOT_CONVERGED
    *_, it, st = O.surfgreen_1985(0.0, h00, h01, 1e-6, itermax=2)
    assert it == 2 and st & O.ST_NOT_CONVERGED


def test_reference_literals():
    assert O.ACCURACY_REF == pytest.approx(1.0000000168623835e-16, rel=0, abs=0)
    assert O.EPS9 == np.float32(1e-9)
    assert O.PI_REF != np.pi and abs(O.PI_REF - np.pi) < 4e-15


def test_reordered_probe_is_a_correct_evaluation():
    """The reordered FP64 evaluation (zgetrf + zgetri inverse, split-K products)
    that measures a point's FP64 noise floor computes the same decimation: it
    meets the closed-form chain and the thick-slab block like the oracle, and
    on a well-conditioned synthetic point it agrees with the oracle to 1e-12."""
    e0, t = 0.3, 1.0
    h00, h01 = chain_h(1, e0, t)
    for w_ev in (-1.0, 0.3, 1.7):
        gll, grr, gb, it, st = O.surfgreen_1985(w_ev * EV, h00, h01, 1e-2 * EV, reordered=True)
        gs, gbk = O.chain_surface_gf(complex(w_ev * EV, 1e-2 * EV), e0 * EV, t * EV)
        assert st == 0 and abs(gll[0, 0] - gs) <= 1e-10 * abs(gs) and abs(gb[0, 0] - gbk) <= 1e-10 * abs(gbk)
    m = synthetic.make_model(6, 2, seed=9)
    top = [1, 2, 3]
    a = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, 6, 2, [[0.1, 0.2]], [0.05], 1e-2 * EV, top, top)
    b = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, 6, 2, [[0.1, 0.2]], [0.05], 1e-2 * EV, top, top,
                           reordered=True)
    for n in ("dos_l", "dos_r", "dos_bulk"):
        assert abs(b[n][0, 0] - a[n][0, 0]) <= 1e-12 * abs(a[n][0, 0])
    assert a["iters"][0, 0] == b["iters"][0, 0]
