"""The drop-in end to end on the reference's own example: the 3D Weyl model's
wt.in-surfacestates (SlabSS_calc and SlabArc_calc, SURFACE card 1 0 0 / 0 0 1)
and its Weyl3D_hr.dat, through the GPU path, to the reference's output files.

Checked against the oracle's pipeline on the same inputs (its own remap of
src/readHmnR.f90:578-766 and its surface spectrum): the raw sums to 1e-9, and
every value read back from dos.dat_l / dos.dat_r / dos.dat_bulk /
spindos.dat_l / spindos.dat_r / arc.dat_* to the oracle's within the files'
own rounding (E16.8 keeps 8 significant digits, F16.8 8 decimals) plus 1e-9
relative; the columns that are differences or spin projections (dos_*_only,
sx / sy / sz) take the 1e-9 relative to the point's spectral densities.  The oracle covers a strided subset of the 201 x 400 spectrum and of
the 201 x 201 plane; the GPU computes them whole."""
import shutil

import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import dropin, hrfile, wtin
from wannier_tools_gb300._lib import PREC_MIXED

from .conftest import GOLDEN

pytestmark = pytest.mark.gpu

A2B = wtin.ANGSTROM2ATOMIC


def _inputs(tmp_path):
    shutil.copy(GOLDEN / "weyl3d_wt.in", tmp_path / "wt.in")
    d = np.load(GOLDEN / "weyl3d_hr_model.npz")
    hrfile.write_hr(tmp_path / "Weyl3D_hr.dat", d["irvec"], d["ndegen"], d["hmnr_ev"],
                    header=" 2-band 3D WSM model")
    return tmp_path / "wt.in"


def _e16_tol(v):
    """Half a unit in the 8th significant digit of E16.8, plus 1e-9 relative."""
    v = np.abs(np.asarray(v, float))
    e = np.floor(np.log10(np.where(v > 0, v, 1.0))) + 1
    return 0.5 * 10.0 ** (e - 8) + 1e-9 * v


def _oracle_model(wt):
    w, geo, _, top, bot = dropin.load_model(wt)
    hr = hrfile.to_hartree(hrfile.read_hr(wt.parent / w.hrfile), w.e_fermi)
    irv, nd, h = O.get_hmnr_cell(hr["irvec"], hr["ndegen"], hr["hmnr"], geo.umatrix,
                                 wtin.orbital_atoms(w.nprojs, w.soc), w.pos_direct, geo.pos_new)
    return w, geo, irv, nd, h, top, bot


def test_dropin_weyl_example(built_lib, tmp_path):
    wt = _inputs(tmp_path)
    out = tmp_path / "out"
    res = dropin.run(wt, out)
    names = sorted(p.name for p in res["files"])
    assert names == sorted(["dos.dat_l", "dos.dat_r", "dos.dat_bulk", "spindos.dat_l", "spindos.dat_r",
                            "arc.dat_l", "arc.dat_r", "arc.dat_bulk"])
    w, geo, irv, nd, h, top, bot = _oracle_model(wt)
    nw = w.num_wann

    # surfstat: 201 k x 400 omega, the oracle on every 40th k point with all omegas
    ss = res["surfstat"]
    assert ss["dos_l"].shape == (201, 400) and (ss["status"] == 0).all()
    kidx = np.arange(0, 201, 40)
    ref = O.surface_spectrum(h, irv, nd, nw, w.np_, ss["k2_path"][kidx], ss["omega"], ss["eta"], top, bot,
                             with_spin=True)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        e = np.abs(ss[name][kidx] - ref[name]) / np.abs(ref[name])
        assert e.max() <= 1e-9, (name, e.max())
    post = dict(zip(("log_dos_l", "log_dos_r", "log_dos_bulk", "dos_l_only", "dos_r_only"),
                    O.surfstat_post(ref["dos_l"], ref["dos_r"], ref["dos_bulk"])))
    scale = {"l": np.abs(ref["dos_l"]) + np.abs(ref["dos_bulk"]),
             "r": np.abs(ref["dos_r"]) + np.abs(ref["dos_bulk"])}
    cols = {"dos.dat_l": (("log_dos_l", None), ("dos_l_only", "l")),
            "dos.dat_r": (("log_dos_r", None), ("dos_r_only", "r")),
            "dos.dat_bulk": (("log_dos_bulk", None),)}
    for fname, keys in cols.items():
        rows = dropin.read_dat(out / fname).reshape(201, 400, -1)[kidx]
        assert np.allclose(rows[:, 0, 0], ss["k2len"][kidx] * A2B, rtol=0, atol=1e-7)   # k (1/Angstrom)
        assert np.allclose(rows[0, :, 1], ss["omega"] / O.EV2HARTREE, rtol=0, atol=1e-7)  # E (eV)
        for c, (key, side) in enumerate(keys):
            got, want = rows[:, :, 2 + c], post[key]
            tol = _e16_tol(want) + (1e-9 * scale[side] if side else 0.0)
            assert (np.abs(got - want) <= tol).all(), (fname, key)
    assert np.isclose(dropin.read_dat(out / "dos.dat_l")[-1, 0], 2 * wtin.PI_REF)   # |Ka2|, 1/Angstrom
    for side in ("l", "r"):
        rows = dropin.read_dat(out / f"spindos.dat_{side}").reshape(201, 400, -1)[kidx]
        s = np.stack([ref[f"s{c}_{side}"] for c in "xyz"], -1) @ geo.urot.T
        for c in range(3):
            tol = _e16_tol(s[:, :, c]) + 1e-9 * scale[side]
            assert (np.abs(rows[:, :, 2 + c] - s[:, :, c]) <= tol).all(), (side, c)

    # SurfaceDOSkk: the 201 x 201 plane at E_arc, the oracle on every 401st point
    arc = res["arc"]
    assert (arc["nkx"], arc["nky"]) == (201, 201) and (arc["status"] == 0).all()
    pidx = np.arange(0, 201 * 201, 401)
    aref = O.surface_spectrum(h, irv, nd, nw, w.np_, arc["k12"][pidx], [w.iso_energy * O.EV2HARTREE],
                              w.fermi_broadening * O.EV2HARTREE, top, bot, scale=1.0 / O.PI_REF)
    for name in ("dos_l", "dos_r", "dos_bulk"):
        e = np.abs(arc[name][pidx, 0] - aref[name][:, 0]) / np.abs(aref[name][:, 0])
        assert e.max() <= 1e-9, (name, e.max())
    for side, name in (("l", "dos_l"), ("r", "dos_r"), ("bulk", "dos_bulk")):
        rows = dropin.read_dat(out / f"arc.dat_{side}")[pidx]
        assert np.allclose(rows[:, :2], arc["k12_shape"][pidx] * A2B, rtol=0, atol=1e-8)
        want = np.log(np.abs(aref[name][:, 0]))
        assert (np.abs(rows[:, 2] - want) <= 0.5e-8 + 1e-9 * np.abs(want)).all(), side


def test_dropin_mixed_form(built_lib, tmp_path):
    """The same run in the split-BF16 form: spectra within 1e-5 of the FP64 run."""
    wt = _inputs(tmp_path)
    a = dropin.run(wt, tmp_path / "fp64")
    b = dropin.run(wt, tmp_path / "mixed", precision=PREC_MIXED)
    for key in ("surfstat", "arc"):
        for name in ("dos_l", "dos_r", "dos_bulk"):
            e = np.abs(b[key][name] - a[key][name]) / np.abs(a[key][name])
            assert e.max() <= 1e-5, (key, name, e.max())
