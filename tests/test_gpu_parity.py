"""GPU parity: libwtgpu.so (through the C ABI) against the CPU oracle.

Tolerance: the plain form is all-FP64 and must match the reference's FP64
LAPACK decimation to a max relative error of 1e-9 in dos_l / dos_r /
dos_bulk; matrices are compared normwise at the same bound."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, synthetic
from wannier_tools_gb300._lib import PT_NOT_CONVERGED

from .conftest import GOLDEN

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE
RTOL = 1e-9


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def nrel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def lib(built_lib):
    return built_lib


def test_device_info(lib):
    info = api.device_info()
    assert "SMs" in info


@pytest.mark.parametrize("nw,np_", [(1, 1), (4, 2), (20, 2), (7, 3), (56, 2)])
def test_ham_qlayer2qlayer_parity(lib, nw, np_):
    m = synthetic.make_model(nw, np_, seed=nw * 10 + np_)
    with api.Model.from_surface_model(m) as g:
        for k in ([0.0, 0.0], [0.1234, -0.4321], [-0.5, 0.5]):
            a00, a01 = g.ham_qlayer2qlayer(k)
            b00, b01 = O.ham_qlayer2qlayer(k, m.hmnr, m.irvec, m.ndegen, nw, np_)
            assert np.abs(a00 - b00).max() <= 1e-13 * np.abs(b00).max()
            assert np.abs(a01 - b01).max() <= 1e-13 * max(np.abs(b01).max(), 1e-30)


def test_ham_ijmax_cut(lib):
    m = synthetic.make_model(3, 3, seed=4)
    with api.Model(m.hmnr, m.irvec, m.ndegen, 3, ijmax=1) as g:
        a00, a01 = g.ham_qlayer2qlayer([0.2, 0.3])
    b00, b01 = O.ham_qlayer2qlayer([0.2, 0.3], m.hmnr, m.irvec, m.ndegen, 3, 3, ijmax=1)
    assert np.allclose(a00, b00, rtol=0, atol=1e-15) and np.allclose(a01, b01, rtol=0, atol=1e-15)


@pytest.mark.parametrize("n", [1, 2, 8, 17, 40, 64, 112])
def test_surfgreen_1985_full_matrices(lib, n):
    nw, np_ = (n // 2, 2) if n % 2 == 0 and n > 2 else (n, 1)
    m = synthetic.make_model(nw, np_, seed=100 + n)
    h00, h01 = O.ham_qlayer2qlayer([0.17, -0.29], m.hmnr, m.irvec, m.ndegen, nw, np_)
    for w_ev, eta_ev in ((0.05, 1e-2), (-0.7, 1e-3)):
        ref = O.surfgreen_1985(w_ev * EV, h00, h01, eta_ev * EV)
        got = api.surfgreen_1985(w_ev * EV, h00, h01, eta_ev * EV)
        for a, b in zip(got[:3], ref[:3]):
            assert nrel(a, b) <= RTOL
        assert abs(got[3] - ref[3]) <= 1
        assert got[4] == ref[4]


def test_chain_closed_form_on_gpu(lib):
    d = np.load(GOLDEN / "analytic_chain.npz")
    m = synthetic.chain_model(float(d["e0_ev"]), float(d["t_ev"]))
    with api.Model.from_surface_model(m) as g:
        for a, eta in enumerate(d["etas"]):
            r = g.surface_spectrum([[0.0, 0.0]], d["omegas"], eta, [1], [1])
            assert rel(r["dos_l"][0], -d["g_surface"][a].imag) <= RTOL
            assert rel(r["dos_r"][0], -d["g_surface"][a].imag) <= RTOL
            assert rel(r["dos_bulk"][0], -d["g_bulk"][a].imag) <= RTOL


def test_golden_weyl3d(lib):
    d = np.load(GOLDEN / "oracle_weyl3d.npz")
    with api.Model(d["hmnr_sc"], d["irvec_sc"], d["ndegen_sc"], int(d["np_"])) as g:
        h00, h01 = g.ham_qlayer2qlayer(d["kpath"][1])
        assert np.abs(h00 - d["h00"]).max() <= 1e-14 and np.abs(h01 - d["h01"]).max() <= 1e-14
        r = g.surface_spectrum(d["kpath"], d["omega"], float(d["eta"]), d["top"], d["bot"])
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert rel(r[name], d[name]) <= RTOL, name
    assert np.abs(r["iters"] - d["iters"]).max() <= 1
    assert (r["status"] == d["status"]).all()


def test_golden_synth_n8(lib):
    d = np.load(GOLDEN / "oracle_synth_n8.npz")
    m = synthetic.make_model(int(d["nw"]), int(d["np_"]), seed=int(d["seed"]))
    with api.Model.from_surface_model(m) as g:
        r = g.surface_spectrum(d["kpts"], d["omega"], float(d["eta"]), d["top"], d["bot"])
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert rel(r[name], d[name]) <= RTOL, name
    h00, h01 = O.ham_qlayer2qlayer(d["kpts"][0], m.hmnr, m.irvec, m.ndegen, 4, 2)
    got = api.surfgreen_1985(d["omega"][2], h00, h01, float(d["eta"]))
    assert nrel(got[0], d["gll"]) <= RTOL and nrel(got[2], d["gb"]) <= RTOL


@pytest.mark.parametrize("nw,np_,eta_ev,arc", [(20, 2, 1e-2, False), (6, 3, 1e-3, True), (56, 2, 1e-3, True)])
def test_spectrum_parity_vs_oracle(lib, nw, np_, eta_ev, arc):
    """Seeded synthetic models of the workload shapes (Ndim 40 / 18 / 112)."""
    m = synthetic.make_model(nw, np_, seed=nw + 17 * np_)
    kp = synthetic.random_kpoints(3 if nw < 50 else 2, seed=nw)
    om = np.array([-0.6, 0.0, 0.45]) * EV if not arc else np.array([0.0]) * EV
    top = list(range(1, nw + 1, 2))
    bot = list(range(2, nw + 1, 3))
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, kp, om, eta_ev * EV, top, bot,
                             scale=(1.0 / O.PI_REF if arc else 1.0))
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum(kp, om, eta_ev * EV, top, bot, divide_by_pi=arc)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert rel(got[name], ref[name]) <= RTOL, name
    assert np.abs(got["iters"] - ref["iters"]).max() <= 1
    assert (got["status"] == ref["status"]).all()


def test_c1_tolerance_and_itermax(lib):
    """Config-1 tolerance (1e-10) and itermax edge cases, flags as the oracle."""
    m = synthetic.make_model(20, 2, seed=1)
    kp = [[0.0, 0.1]]
    om = np.array([-0.3, 0.2]) * EV
    with api.Model.from_surface_model(m) as g:
        for tol, itmax in ((1e-10, 100), (1e-16, 3), (1e-16, 0)):
            ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, 20, 2, kp, om, 1e-2 * EV, [1, 2], [3],
                                     accuracy=tol, itermax=itmax)
            got = g.surface_spectrum(kp, om, 1e-2 * EV, [1, 2], [3], tol=tol, itermax=itmax)
            for name in ("dos_l", "dos_r", "dos_bulk"):
                assert rel(got[name], ref[name]) <= RTOL
            assert (got["status"] == ref["status"]).all()
            if itmax < 10:
                assert (got["status"] & PT_NOT_CONVERGED).all()
                assert (got["iters"] == itmax).all()


def test_empty_and_ragged_inputs(lib):
    m = synthetic.make_model(3, 2, seed=8)
    with api.Model.from_surface_model(m) as g:
        r = g.surface_spectrum(np.zeros((0, 2)), [0.0], 1e-3, [1], [1])
        assert r["dos_l"].shape == (0, 1)
        r = g.surface_spectrum([[0.1, 0.1]], [], 1e-3, [1], [1])
        assert r["dos_l"].shape == (1, 0)
        # no orbitals listed: surface sums are zero, bulk still computed
        r = g.surface_spectrum([[0.1, 0.1], [0.2, -0.3]], [0.0, 0.01], 1e-3, [], [])
        assert (r["dos_l"] == 0).all() and (r["dos_r"] == 0).all() and (r["dos_bulk"] > 0).all()


def test_bad_arguments_raise(lib):
    from wannier_tools_gb300._lib import WtgError
    m = synthetic.make_model(3, 1, seed=8)
    with api.Model.from_surface_model(m) as g:
        with pytest.raises(WtgError):
            g.surface_spectrum([[0.1, 0.1]], [0.0], 1e-3, [4], [1])       # orbital > nw
        with pytest.raises(WtgError):
            g.surface_spectrum([[0.1, 0.1]], [0.0], 1e-3, [1], [1], itermax=-1)


def test_ndim_limits(lib):
    """Ndim 118 runs the shared-memory inverse, Ndim 122 the global-memory one;
    both match the oracle.  Ndim 322 is beyond the largest supported (320)."""
    from wannier_tools_gb300._lib import WtgError
    for nw in (59, 61):
        m = synthetic.make_model(nw, 2, seed=3)
        with api.Model.from_surface_model(m) as g:
            r = g.surface_spectrum([[0.3, 0.3]], [0.02 * EV], 1e-2 * EV, [1], [1])
        ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, 2, [[0.3, 0.3]], [0.02 * EV],
                                 1e-2 * EV, [1], [1])
        for name in ("dos_l", "dos_r", "dos_bulk"):
            assert rel(r[name], ref[name]) <= RTOL, (nw, name)
    m = synthetic.make_model(161, 2, seed=3)
    with api.Model.from_surface_model(m) as g:
        with pytest.raises(WtgError):
            g.surface_spectrum([[0.3, 0.3]], [0.0], 1e-2, [1], [1])


def test_many_points_properties(lib):
    """A larger batch (more instances than resident CTAs): positivity, the
    k -> -k symmetry of a time-reversal-free but Hermitian model is not
    assumed; instead results must not depend on batch composition."""
    m = synthetic.make_model(10, 2, seed=12)
    kp = synthetic.random_kpoints(64, seed=1)
    om = np.linspace(-1, 1, 25) * EV
    with api.Model.from_surface_model(m) as g:
        full = g.surface_spectrum(kp, om, 1e-2 * EV, [1, 2, 3], [4, 5])
        part = g.surface_spectrum(kp[10:13], om[5:9], 1e-2 * EV, [1, 2, 3], [4, 5])
    assert (full["dos_bulk"] > 0).all() and (full["dos_l"] > 0).all()
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert np.array_equal(full[name][10:13, 5:9], part[name])


@pytest.mark.parametrize("nw,np_,arc", [(6, 2, False), (6, 2, True), (5, 1, False), (10, 3, True)])
def test_spin_resolved_spectra(lib, nw, np_, arc):
    """sx/sy/sz of GLL and GRR (src/surfstat.f90:162-192, src/fermiarc.f90:250-330)
    against the oracle's six full products with the Pauli matrices."""
    m = synthetic.make_model(nw, np_, seed=50 + nw)
    kp = synthetic.random_kpoints(2, seed=nw)
    om = np.array([-0.2, 0.35]) * EV
    top = [1, 2, nw]
    bot = [1, (nw + 1) // 2]
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, kp, om, 1e-2 * EV, top, bot,
                             scale=(1.0 / O.PI_REF if arc else 1.0), with_spin=True)
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum_spin(kp, om, 1e-2 * EV, top, bot, arc=arc)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert rel(got[name], ref[name]) <= RTOL, name
    for name in ("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r"):
        scale = np.abs(ref["dos_l"]).max()
        assert np.max(np.abs(got[name] - ref[name])) <= 1e-9 * scale, name


def test_fp64_throughput_probes(built_lib):
    """The live roofline denominators: DFMA and DMMA rates are positive and of the
    order of a GB300's FP64 rate (about 1.2 TFLOP/s)."""
    dfma, dmma = api.fp64_peak_tflops(), api.dmma_peak_tflops()
    print("FP64 DFMA %.3f TFLOP/s, DMMA %.3f TFLOP/s" % (dfma, dmma))
    assert 0.2 < dfma < 20 and 0.2 < dmma < 20
