"""Writers of the reference's output files (dos.dat_*, spindos.dat_*, arc.dat_*):
Fortran edit-descriptor formatting and the files' layout, on CPU."""
import numpy as np
import pytest

from wannier_tools_gb300 import outfiles
from wannier_tools_gb300.api import EPS9


@pytest.mark.parametrize("v,s", [
    (1.5, "  0.15000000E+01"),
    (-2.5e-10, " -0.25000000E-09"),
    (0.0, "  0.00000000E+00"),
    (123456789.0, "  0.12345679E+09"),
    (9.999999999, "  0.10000000E+02"),
    (1e100, "  0.10000000+101"),
    (-3.0e-120, " -0.30000000-119"),
    (float("nan"), "             NaN"),
    (float("-inf"), "       -Infinity"),
])
def test_fortran_e16_8(v, s):
    assert outfiles.fortran_e(v) == s
    assert len(outfiles.fortran_e(v)) == 16


def test_fortran_f16_8():
    assert outfiles.fortran_f(0.5) == "      0.50000000"
    assert outfiles.fortran_f(-1e-10) == "     -0.00000000"
    assert outfiles.fortran_f(1e12) == "*" * 16
    assert outfiles.fortran_f(float("-inf")) == "       -Infinity"


def test_surfstat_files(tmp_path):
    rng = np.random.default_rng(3)
    nk, nom = 3, 4
    dl = rng.uniform(0.1, 2.0, (nk, nom))
    dr = rng.uniform(0.1, 2.0, (nk, nom))
    db = rng.uniform(0.1, 2.0, (nk, nom))
    klen = np.linspace(0, 0.5, nk)
    om = np.linspace(-0.02, 0.02, nom)
    spin = {f"s{c}_{s}": rng.normal(size=(nk, nom)) for c in "xyz" for s in "lr"}
    rot = np.array([[0, 1, 0], [-1, 0, 0], [0, 0, 1.0]])
    files = outfiles.write_surfstat(tmp_path, klen, om, dl, dr, db, spin=spin, rotation=rot)
    assert [f.name for f in files] == ["dos.dat_l", "dos.dat_r", "dos.dat_bulk",
                                       "spindos.dat_l", "spindos.dat_r"]
    text = (tmp_path / "dos.dat_l").read_text().split("\n")
    assert text[0] == "#" + " k(1/Ang)".rjust(12) + " E(eV)".rjust(17) + "dos_l".rjust(17) + "dos_l_only".rjust(17)
    assert text[1 + nom] == ""                      # blank record after each k point
    a = np.loadtxt(tmp_path / "dos.dat_l")
    assert a.shape == (nk * nom, 4)
    np.testing.assert_allclose(a[:, 0], np.repeat(klen * outfiles.ANGSTROM2ATOMIC, nom), rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(a[:, 1], np.tile(om * 27.211385, nk), rtol=1e-7)
    np.testing.assert_allclose(a[:, 2], np.log(dl).ravel(), rtol=1e-7)
    only = np.where(dl - db < 0, EPS9, dl - db).ravel()
    np.testing.assert_allclose(a[:, 3], only, rtol=1e-7)
    b = np.loadtxt(tmp_path / "dos.dat_bulk")
    np.testing.assert_allclose(b[:, 2], np.log(db + EPS9).ravel(), rtol=1e-7)
    sp = np.loadtxt(tmp_path / "spindos.dat_r")
    s = np.stack([spin[f"s{c}_r"] for c in "xyz"], -1).reshape(-1, 3) @ rot.T
    np.testing.assert_allclose(sp[:, 2:], s, rtol=1e-7, atol=1e-12)


def test_surfstat_phonon_energies(tmp_path):
    om2 = np.array([0.01, 0.04]) ** 2
    outfiles.write_surfstat(tmp_path, [0.0], om2, np.ones((1, 2)), np.ones((1, 2)), np.ones((1, 2)),
                            particle="phonon")
    a = np.loadtxt(tmp_path / "dos.dat_r")
    np.testing.assert_allclose(a[:, 1], np.array([0.01, 0.04]) * 27.211385, rtol=1e-7)


def test_arc_files(tmp_path):
    nkx, nky = 3, 5
    rng = np.random.default_rng(4)
    kxy = rng.uniform(-0.3, 0.3, (nkx * nky, 2))
    dl, dr, db = (rng.uniform(0.01, 1.0, nkx * nky) for _ in range(3))
    db[2] = -db[2]
    files = outfiles.write_arc(tmp_path, kxy, dl, dr, db, nky)
    assert [f.name for f in files] == ["arc.dat_l", "arc.dat_r", "arc.dat_bulk"]
    lines = (tmp_path / "arc.dat_bulk").read_text().split("\n")
    assert lines[0] == lines[1]                    # written twice, as the reference does
    assert lines[6] == "#kx".rjust(16) + "ky".rjust(16) + "log(dos)".rjust(16)
    a = np.loadtxt(tmp_path / "arc.dat_bulk")
    assert a.shape == (nkx * nky, 3)
    np.testing.assert_allclose(a[:, :2], kxy * outfiles.ANGSTROM2ATOMIC, atol=1e-8)
    np.testing.assert_allclose(a[:, 2], np.log(np.abs(db)), atol=1e-8)
    body = (tmp_path / "arc.dat_l").read_text().split("\n")[6:]
    assert body[nky].strip() == ""                 # a blank record after every nky points
