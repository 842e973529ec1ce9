"""Mixed-precision form: split-BF16 products on the tcgen05 tensor cores.

Checked against numpy (products, inverses) and against the FP64 oracle
(spectra).  Tolerances: a split product keeps 49 bits per operand against a
per-row / per-column exponent, with every slice order up to 6 summed exactly,
so products must match to 5e-13 normwise (about 6e-14 measured);
Newton-Schulz-refined inverses to 1e-9 normwise; the surface / bulk spectral
densities to the 1e-5 relative error the mixed form is specified for (about
1e-7 typical, a few 1e-6 at the hardest points of the Fermi-arc plane)."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, synthetic
from wannier_tools_gb300._lib import PREC_FP64, PREC_MIXED

pytestmark = pytest.mark.gpu

EV = O.EV2HARTREE


def crand(rng, n, m=None):
    m = m or n
    return rng.normal(size=(n, m)) + 1j * rng.normal(size=(n, m))


def nrel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [1, 8, 17, 40, 64, 112, 130, 200, 257, 320])
def test_mat_mul_both_precisions(built_lib, n):
    rng = np.random.default_rng(n)
    a, b = crand(rng, n), crand(rng, n)
    ref = a @ b
    assert nrel(api.mat_mul(a, b, PREC_FP64), ref) <= 1e-14
    assert nrel(api.mat_mul(a, b, PREC_MIXED), ref) <= 5e-13


def test_mat_mul_mixed_wide_dynamic_range(built_lib):
    """Rows of A and columns of B scaled over 1e-12..1e12: each output element
    keeps its accuracy relative to its own row/column scale."""
    rng = np.random.default_rng(5)
    n = 48
    ra = 10.0 ** rng.uniform(-12, 12, n)
    cb = 10.0 ** rng.uniform(-12, 12, n)
    a = crand(rng, n) * ra[:, None]
    b = crand(rng, n) * cb[None, :]
    got = api.mat_mul(a, b, PREC_MIXED)
    ref = a @ b
    scale = np.outer(ra, cb) * n
    assert np.max(np.abs(got - ref) / scale) <= 1e-10


@pytest.mark.parametrize("n", [1, 5, 40, 112, 113, 200, 264, 320])
def test_inverse_both_precisions(built_lib, n):
    rng = np.random.default_rng(100 + n)
    a = crand(rng, n) + 3.0 * np.sqrt(n) * np.eye(n)
    ref = np.linalg.inv(a)
    g64, st64 = api.inv(a, PREC_FP64)
    assert st64 == 0 and nrel(g64, ref) <= 1e-13
    gmx, stmx = api.inv(a, PREC_MIXED)
    assert stmx == 0 and nrel(gmx, ref) <= 1e-9


def test_inverse_near_pole(built_lib):
    """w - H00 one micro-Hartree from an eigenvalue, eta = 1e-4 eV (condition ~1e6)."""
    m = synthetic.make_model(20, 2, seed=3)
    h00, _ = O.ham_qlayer2qlayer([0.1, 0.2], m.hmnr, m.irvec, m.ndegen, 20, 2)
    ev = np.linalg.eigvalsh(h00)
    w = complex(ev[17] + 1e-6, 1e-4 * EV)
    a = w * np.eye(40) - h00
    ref = np.linalg.inv(a)
    gmx, st = api.inv(a, PREC_MIXED)
    # split products good to ~1e-14 normwise: error well below 1e-12 x condition number (~1e6 here)
    assert st == 0 and nrel(gmx, ref) <= 1e-12 * np.linalg.cond(a)


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


@pytest.mark.parametrize("nw,np_,eta_ev,oms,arc", [
    (20, 2, 1e-2, [-0.6, 0.0, 0.45], False),    # surfstat shape, Ndim 40
    (56, 2, 1e-3, [0.0], True),                  # Fermi-arc shape, Ndim 112
    (8, 2, 1e-4, [0.0, 0.7], False),             # small eta, Ndim 16
    (44, 3, 1e-3, [0.05], False),                # Np = 3, Ndim 132: two row blocks
    (88, 3, 1e-3, [-0.2], False),                # Ndim 264: six accumulators, three row blocks
])
def test_spectrum_mixed_vs_fp64_oracle(built_lib, nw, np_, eta_ev, oms, arc):
    m = synthetic.make_model(nw, np_, seed=nw + np_)
    kp = synthetic.random_kpoints(3 if nw * np_ <= 132 else 2, seed=nw)
    om = np.asarray(oms) * EV
    top = list(range(1, nw + 1, 2))
    bot = list(range(2, nw + 1, 3))
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum(kp, om, eta_ev * EV, top, bot, divide_by_pi=arc,
                                 precision=PREC_MIXED)
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, kp, om, eta_ev * EV, top, bot,
                             scale=(1.0 / O.PI_REF if arc else 1.0))
    errs = {name: _rel(got[name], ref[name]) for name in ("dos_l", "dos_r", "dos_bulk")}
    print("mixed max rel err", nw, np_, eta_ev, errs)
    for name, e in errs.items():
        assert e <= 1e-5, (name, e)
    assert np.abs(got["iters"] - ref["iters"]).max() <= 1
    assert (got["status"] == 0).all()


def test_mixed_ndim_limit(built_lib):
    from wannier_tools_gb300._lib import WtgError
    m = synthetic.make_model(161, 2, seed=3)
    with api.Model.from_surface_model(m) as g:
        with pytest.raises(WtgError):
            g.surface_spectrum([[0.3, 0.3]], [0.0], 1e-2, [1], [1], precision=PREC_MIXED)


def test_spin_mixed(built_lib):
    nw, np_ = 8, 2
    m = synthetic.make_model(nw, np_, seed=77)
    kp = synthetic.random_kpoints(2, seed=3)
    om = np.array([0.1]) * EV
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, kp, om, 1e-2 * EV, [1, 2, 5],
                             [1, 4], scale=1.0 / O.PI_REF, with_spin=True)
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum_spin(kp, om, 1e-2 * EV, [1, 2, 5], [1, 4], arc=True,
                                      precision=PREC_MIXED)
    scale = np.abs(ref["dos_l"]).max()
    for name in ("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r"):
        assert np.max(np.abs(got[name] - ref[name])) <= 1e-6 * scale, name


@pytest.mark.parametrize("arc", [False, True])
def test_spin_mixed_ndim132(built_lib, arc):
    """Ndim 132 (Np 3): GLL and GRR come from Schur complements eliminated in
    global memory (GRR in full where surfstat's spin sums read its top block)."""
    nw, np_ = 44, 3
    m = synthetic.make_model(nw, np_, seed=78)
    kp = synthetic.random_kpoints(2, seed=4)
    om = np.array([0.05]) * EV
    top, bot = [1, 2, 5, 23, 40], [1, 3, 24, 44]
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, kp, om, 1e-3 * EV, top, bot,
                             scale=1.0 / O.PI_REF if arc else 1.0, with_spin=True)
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum_spin(kp, om, 1e-3 * EV, top, bot, arc=arc, precision=PREC_MIXED)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        assert _rel(got[name], ref[name]) <= 1e-5, name
    scale = np.abs(ref["dos_l"]).max()
    for name in ("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r"):
        assert np.max(np.abs(got[name] - ref[name])) <= 1e-5 * scale, name


def _oracle_point(args):
    from oracle import wt_oracle as Ow
    from wannier_tools_gb300 import synthetic as S
    nw, np_, seed, k, om, eta = args
    m = S.make_model(nw, np_, seed=seed)
    top = list(range(1, nw + 1))
    r = Ow.surface_spectrum(m.hmnr, m.irvec, m.ndegen, nw, np_, k, om, eta, top, top,
                            scale=1.0 / Ow.PI_REF)
    return {n: r[n] for n in ("dos_l", "dos_r", "dos_bulk", "iters")}


def test_spectrum_mixed_arc_plane_dense(built_lib):
    """192 points spread over the 201 x 201 Fermi-arc plane of the Ndim = 112
    model (eta = 1e-3 eV, every orbital in both lists): every point within
    1e-5 of the FP64 oracle.  Points near poles need more than one in-loop
    refinement step; a fixed single step leaves errors near 3e-4 here."""
    import multiprocessing as mp
    import os
    nw, np_, seed, eta = 56, 2, 2024, 1e-3 * EV
    _, _, kall = api.kplane_slab(201, 201, (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    idx = np.arange(192) * (len(kall) // 192)
    kp = kall[idx]
    om = np.array([0.0])
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        parts = pool.map(_oracle_point, [(nw, np_, seed, kp[[i]], om, eta) for i in range(len(kp))])
    ref = {n: np.concatenate([p[n] for p in parts]) for n in ("dos_l", "dos_r", "dos_bulk", "iters")}
    m = synthetic.make_model(nw, np_, seed=seed)
    top = list(range(1, nw + 1))
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum(kp, om, eta, top, top, divide_by_pi=True, precision=PREC_MIXED)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        e = _rel(got[name].ravel(), ref[name].ravel())
        print("dense arc plane", name, e)
        assert e <= 1e-5, (name, e)
    assert (got["status"] == 0).all()


# The 24 points of the 201 x 201 Fermi-arc plane of the Ndim = 112 model where the
# mixed form differed most from the FP64 form when the slice orders 6, 7 and 8
# shared one truncating accumulator (1e-5 to 4.3e-5, over the whole plane solved
# in both forms).  There two valid FP64 evaluations already differ by ~1e-7: the
# points amplify rounding about 1e9-fold.
HARD_ARC_POINTS = [746, 1658, 1964, 2798, 9751, 14653, 14861, 15272, 18819, 19743, 24760, 25019,
                   27245, 27540, 28495, 29241, 29881, 31184, 31622, 32239, 32435, 33251, 33710,
                   37089]


def test_spectrum_mixed_hardest_arc_points(built_lib):
    """The mixed form within 1e-5 of the FP64 oracle at the plane's hardest points."""
    import multiprocessing as mp
    import os
    nw, np_, seed, eta = 56, 2, 2024, 1e-3 * EV
    _, _, kall = api.kplane_slab(201, 201, (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    kp = kall[HARD_ARC_POINTS]
    om = np.array([0.0])
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        parts = pool.map(_oracle_point, [(nw, np_, seed, kp[[i]], om, eta) for i in range(len(kp))])
    ref = {n: np.concatenate([p[n] for p in parts]) for n in ("dos_l", "dos_r", "dos_bulk", "iters")}
    m = synthetic.make_model(nw, np_, seed=seed)
    top = list(range(1, nw + 1))
    with api.Model.from_surface_model(m) as g:
        got = g.surface_spectrum(kp, om, eta, top, top, divide_by_pi=True, precision=PREC_MIXED)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        e = _rel(got[name].ravel(), ref[name].ravel())
        print("hardest arc points", name, e)
        assert e <= 1e-5, (name, e)
    assert np.abs(got["iters"].ravel() - ref["iters"].ravel()).max() <= 1


def _whole_configuration(nw, np_, seed, kpts, om, eta, tol, divide_by_pi):
    m = synthetic.make_model(nw, np_, seed=seed)
    top = list(range(1, nw + 1))
    with api.Model.from_surface_model(m) as g:
        ref = g.surface_spectrum(kpts, om, eta, top, top, tol=tol, divide_by_pi=divide_by_pi,
                                 precision=PREC_FP64)
        got = g.surface_spectrum(kpts, om, eta, top, top, tol=tol, divide_by_pi=divide_by_pi,
                                 precision=PREC_MIXED)
    assert (ref["status"] == 0).all() and (got["status"] == 0).all()
    assert np.abs(got["iters"] - ref["iters"]).max() <= 1
    return {name: _rel(got[name].ravel(), ref[name].ravel()) for name in ("dos_l", "dos_r", "dos_bulk")}


def test_mixed_whole_kpath_ndim40(built_lib):
    """Every point of the Ndim-40 k-path x omega spectrum (101 k x 201 omega in
    [-1, 1] eV, eta 1e-2 eV, tol 1e-10): the mixed form within 1e-5 of the FP64 form."""
    kp = api.kpath_slab([((-0.5, 0.0), (0.5, 0.0))], 101)
    om = np.linspace(-1.0, 1.0, 201) * EV
    errs = _whole_configuration(20, 2, 2023, kp, om, 1e-2 * EV, 1e-10, False)
    print("whole Ndim-40 k-path", errs)
    for name, e in errs.items():
        assert e <= 1e-5, (name, e)


def test_mixed_whole_arc_plane_ndim112(built_lib):
    """Every point of the 201 x 201 Fermi-arc plane of the Ndim-112 model (omega 0,
    eta 1e-3 eV, every orbital in both lists, /pi): the mixed form within 1e-5 of the
    FP64 form (3.6e-6 measured), including the points where two valid FP64
    evaluations already differ by ~1e-7."""
    _, _, kall = api.kplane_slab(201, 201, (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    errs = _whole_configuration(56, 2, 2024, kall, np.array([0.0]), 1e-3 * EV, O.ACCURACY_REF, True)
    print("whole arc plane", errs)
    for name, e in errs.items():
        assert e <= 1e-5, (name, e)
