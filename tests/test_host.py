"""Host-side logic on CPU: synthetic models, hr.dat I/O and the surface-cell
remap, grids and output transforms, each against the oracle's restatement."""
import numpy as np

from oracle import wt_oracle as O
from wannier_tools_gb300 import api, hrfile, synthetic

from .conftest import GOLDEN


def test_synthetic_model_is_hermitian_and_seeded():
    m = synthetic.make_model(5, 2, seed=3)
    assert m.nrpts == 343 and m.hmnr.shape == (343, 5, 5)
    idx = {tuple(r): i for i, r in enumerate(m.irvec)}
    for i, r in enumerate(m.irvec):
        j = idx[(-r[0], -r[1], -r[2])]
        assert np.array_equal(m.hmnr[j], m.hmnr[i].conj().T)
    # R1 fastest, then R2, then R3 (the surface-cell order of get_hmnr_cell)
    assert list(m.irvec[0]) == [-3, -3, -3] and list(m.irvec[1]) == [-2, -3, -3]
    assert list(m.irvec[7]) == [-3, -2, -3]
    m2 = synthetic.make_model(5, 2, seed=3)
    assert np.array_equal(m.hmnr, m2.hmnr)
    onsite = np.diag(m.hmnr[idx[(0, 0, 0)]]).real / synthetic.EV2HARTREE
    assert (np.abs(onsite) <= 1.0).all()


def test_hr_roundtrip_and_surface_cell(tmp_path):
    d = np.load(GOLDEN / "weyl3d_hr_model.npz")
    p = tmp_path / "w_hr.dat"
    hrfile.write_hr(p, d["irvec"], d["ndegen"], d["hmnr_ev"])
    hr = hrfile.read_hr(p)
    assert np.array_equal(hr["irvec"], d["irvec"])
    assert np.allclose(hr["hmnr"], d["hmnr_ev"], atol=1e-8)
    hh = hrfile.to_hartree(hr, e_fermi_ev=0.5)
    r0 = [i for i, r in enumerate(hr["irvec"]) if tuple(r) == (0, 0, 0)][0]
    assert np.allclose(np.diag(hh["hmnr"][r0]), (np.diag(hr["hmnr"][r0]) - 0.5) * O.EV2HARTREE)
    sc = hrfile.surface_cell(hh)
    irv, nd, h = O.get_hmnr_cell_identity(hh["irvec"], hh["ndegen"], hh["hmnr"])
    assert np.array_equal(sc["irvec"], irv) and np.array_equal(sc["ndegen"], nd)
    assert np.array_equal(sc["hmnr"], h)


def test_surface_cell_shuffled_and_cut():
    m = synthetic.make_model(2, 1, seed=4)
    rng = np.random.default_rng(0)
    perm = rng.permutation(m.nrpts)
    irv = m.irvec[perm].copy()
    irv[0] = [9, 0, 0]                                   # beyond max_ir = 8: dropped
    nd = rng.integers(1, 4, m.nrpts).astype(np.int32)
    hr = {"irvec": irv, "ndegen": nd, "hmnr": m.hmnr[perm]}
    sc = hrfile.surface_cell(hr)
    o_irv, o_nd, o_h = O.get_hmnr_cell_identity(irv, nd, m.hmnr[perm])
    assert np.array_equal(sc["irvec"], o_irv) and np.allclose(sc["hmnr"], o_h, rtol=0, atol=0)
    assert sc["irvec"].shape[0] == m.nrpts - 1


def test_grids_match_oracle():
    nkx, nky, k = api.kplane_slab(200, 201, (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    onx, ony, ok, _ = O.kplane_grid(200, 201, (-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    assert (nkx, nky) == (onx, ony) == (201, 201)
    assert np.array_equal(k, ok)
    w, eta = api.surfstat_grid(-1.0, 1.0, 200)
    ow, oeta = O.surfstat_grid(-1.0, 1.0, 200)
    assert np.array_equal(w, ow) and eta == oeta
    assert w[-1] < 1.0                                     # omega excludes OmegaMax
    kp = api.kpath_slab([((-0.5, 0.0), (0.5, 0.0)), ((0.5, 0.0), (0.5, 0.5))], 11)
    assert kp.shape == (22, 2) and np.allclose(kp[10], kp[11])   # repeated segment end


def test_output_transforms_match_oracle():
    rng = np.random.default_rng(1)
    dl, dr, db = (rng.uniform(0.01, 5, (4, 6)) for _ in range(3))
    a = api.surfstat_post(dl, dr, db)
    b = O.surfstat_post(dl, dr, db)
    for x, name in zip(b, ("log_dos_l", "log_dos_r", "log_dos_bulk", "dos_l_only", "dos_r_only")):
        assert np.array_equal(a[name], x)
    for x, y in zip(api.arc_post(dl, dr), O.arc_post(dl, dr)):
        assert np.array_equal(x, y)
