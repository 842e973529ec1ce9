"""The reference's output files of the surface-state path, written from the
drop-in's results so that a run without Fortran leaves the same files behind.

* ``write_surfstat``: dos.dat_l / dos.dat_r / dos.dat_bulk (and spindos.dat_l /
  spindos.dat_r when spin sums are given) of surfstat, ``src/surfstat.f90:270-317``:
  k-path length in 1/Angstrom, energy in eV, log|dos| and the surface-only dos,
  records 4(1X,E16.8) / 3(1X,E16.8) / 5(1X,E16.8), a blank line after each k point.
* ``write_arc``: arc.dat_l / arc.dat_r / arc.dat_bulk of SurfaceDOSkk,
  ``src/fermiarc.f90:419-453``: the same comment header, records (30f16.8) of kx, ky
  (1/Angstrom) and log(dos) (log|dos| for the bulk), a blank record after every nky
  points.

Inputs are what the library returns (raw sums in Hartree units; ``api.surfstat_post``
does the log / _only step of ``src/surfstat.f90:237-247``).  Number formatting follows
the Fortran edit descriptors (``fortran_e``), so the files match the reference's
digit for digit for the same values.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from .api import EPS9, surfstat_post

ANGSTROM2ATOMIC = 1.0 / 0.529177210903      # src/module.f90:711
EV2HARTREE = 1.0 / 27.211385                # src/module.f90:713


def fortran_e(v: float, w: int = 16, d: int = 8) -> str:
    """One value in the Fortran Ew.d edit descriptor: 0.ddddddddE+ee (mantissa in
    [0.1, 1)), right-justified in w columns; three-digit exponents drop the E as
    Fortran does (0.dddddddd+100)."""
    v = float(v)
    if math.isnan(v):
        return "NaN".rjust(w)
    if math.isinf(v):
        return ("-Infinity" if v < 0 else "Infinity").rjust(w)
    if v == 0.0:
        body, e = "0." + "0" * d, 0
    else:
        # round to d significant digits with Python's exact decimal formatting, then
        # shift the decimal point: x.xxxxxxxE+ee -> 0.xxxxxxxxE+(ee+1)
        m, ex = f"{abs(v):.{d - 1}e}".split("e")
        digits = m.replace(".", "")
        body, e = "0." + digits, int(ex) + 1
    sign = "-" if v < 0 or (v == 0.0 and math.copysign(1.0, v) < 0) else ""
    if abs(e) <= 99:
        exp = f"E{'+' if e >= 0 else '-'}{abs(e):02d}"
    else:
        exp = f"{'+' if e >= 0 else '-'}{abs(e):03d}"
    s = sign + body + exp
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_f(v: float, w: int = 16, d: int = 8) -> str:
    """One value in the Fortran Fw.d edit descriptor (Infinity / NaN spelled as
    Fortran writes them; asterisks when the number does not fit)."""
    v = float(v)
    if math.isnan(v):
        return "NaN".rjust(w)
    if math.isinf(v):
        return ("-Infinity" if v < 0 else "Infinity").rjust(w)
    s = f"{v:.{d}f}"
    return s.rjust(w) if len(s) <= w else "*" * w


def _rec(values, w: int = 16, d: int = 8) -> str:
    return "".join(" " + fortran_e(v, w, d) for v in values) + "\n"


def _hdr(first: str, rest) -> str:
    """'("#", a12, 6a17)': '#', the first label right-justified in 12, the others in 17."""
    return "#" + first.rjust(12) + "".join(x.rjust(17) for x in rest) + "\n"


def write_surfstat(outdir, klen, omega, dos_l, dos_r, dos_bulk, spin=None, rotation=None,
                   particle: str = "electron") -> list[Path]:
    """surfstat's files from raw sums.

    klen[nk]               k-path length (1/Bohr; k2len of the reference)
    omega[nomega]          energies in Hartree (for phonons: the squared energies the
                           decimation ran at; the file shows their square roots)
    dos_l/dos_r/dos_bulk   (nk, nomega) raw sums as the library returns them
    spin                   optional dict sx_l, sy_l, sz_l, sx_r, sy_r, sz_r of (nk, nomega)
    rotation               3x3 matrix applied to (sx, sy, sz) before writing (the
                           reference's rotate to the SURFACE frame); identity if None
    """
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    klen = np.asarray(klen, dtype=np.float64).ravel()
    om = np.asarray(omega, dtype=np.float64).ravel()
    if "phonon" in particle:
        om = np.sqrt(om)                                   # src/surfstat.f90:262-267
    post = surfstat_post(np.asarray(dos_l), np.asarray(dos_r), np.asarray(dos_bulk))
    nk, nom = post["log_dos_l"].shape
    if klen.shape[0] != nk or om.shape[0] != nom:
        raise ValueError("klen / omega do not match the dos arrays")
    kx = klen * ANGSTROM2ATOMIC
    ev = om / EV2HARTREE
    files = [out / "dos.dat_l", out / "dos.dat_r", out / "dos.dat_bulk"]
    with open(files[0], "w") as fl, open(files[1], "w") as fr, open(files[2], "w") as fb:
        fl.write(_hdr(" k(1/Ang)", [" E(eV)", "dos_l", "dos_l_only"]))
        fr.write(_hdr(" k(1/Ang)", [" E(eV)", "dos_r", "dos_r_only"]))
        fb.write(_hdr(" k(1/Ang)", [" E(eV)", "dos_bulk"]))
        for i in range(nk):
            for j in range(nom):
                fl.write(_rec((kx[i], ev[j], post["log_dos_l"][i, j], post["dos_l_only"][i, j])))
                fr.write(_rec((kx[i], ev[j], post["log_dos_r"][i, j], post["dos_r_only"][i, j])))
                fb.write(_rec((kx[i], ev[j], post["log_dos_bulk"][i, j])))
            for f in (fl, fr, fb):
                f.write("\n")
    if spin is not None:
        rot = np.eye(3) if rotation is None else np.asarray(rotation, dtype=np.float64)
        for side in ("l", "r"):
            path = out / f"spindos.dat_{side}"
            s = np.stack([np.asarray(spin[f"s{c}_{side}"], dtype=np.float64) for c in "xyz"], -1)
            s = s @ rot.T
            with open(path, "w") as f:
                f.write(f"# spin dos_{side}, the axis is rotated as \n")
                f.write("# x is along R1', z is along R1'xR2', y is along z x y\n")
                f.write(_hdr(" k(1/Ang)", [" E(eV)", "sx", "sy", "sz"]))
                for i in range(nk):
                    for j in range(nom):
                        f.write(_rec((kx[i], ev[j], *s[i, j])))
                    f.write("\n")
            files.append(path)
    return files


_ARC_FRAME = ["# The coordinate of k is redefined according to the SURFACE card\n",
              "# x axis is parallel to R1'\n",
              "# z axis is parallel to R1'xR2'\n",
              "# y axis is parallel to z x x\n"]


def write_arc(outdir, kxy, dos_l, dos_r, dos_bulk, nky: int) -> list[Path]:
    """SurfaceDOSkk's files from raw sums (already divided by pi, as the library
    returns them with divide_by_pi).

    kxy[nkx*nky, 2]        Cartesian in-plane k of each point in the plane's ikp order
                           (1/Bohr; k12_shape of the reference)
    dos_l/dos_r/dos_bulk   nkx*nky values in the same order
    nky                    points per blank-record block (the second k index)
    """
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    k = np.asarray(kxy, dtype=np.float64).reshape(-1, 2) * ANGSTROM2ATOMIC
    with np.errstate(divide="ignore", invalid="ignore"):   # log of a non-positive sum: -Inf / NaN, as Fortran
        vals = {"l": np.log(np.asarray(dos_l, dtype=np.float64).ravel()),
                "r": np.log(np.asarray(dos_r, dtype=np.float64).ravel()),
                "bulk": np.log(np.abs(np.asarray(dos_bulk, dtype=np.float64).ravel()))}
    bulk_line = "#Density of states of bulk system after projection onto the surface BZ\n"
    heads = {"l": ["# Surface density of states of bottom surface\n"],
             "r": ["# Surface density of states of top surface\n"],
             "bulk": [bulk_line, bulk_line]}       # the reference writes this line twice
    files = []
    for side in ("l", "r", "bulk"):
        if vals[side].shape[0] != k.shape[0]:
            raise ValueError("kxy does not match the dos arrays")
        path = out / f"arc.dat_{side}"
        with open(path, "w") as f:
            for line in heads[side] + _ARC_FRAME:
                f.write(line)
            f.write("#kx".rjust(16) + "ky".rjust(16) + "log(dos)".rjust(16) + "\n")
            for ikp in range(k.shape[0]):
                f.write(fortran_f(k[ikp, 0]) + fortran_f(k[ikp, 1]) + fortran_f(vals[side][ikp]) + "\n")
                if (ikp + 1) % nky == 0:
                    f.write("  \n")
        files.append(path)
    return files


__all__ = ["fortran_e", "fortran_f", "write_surfstat", "write_arc", "EPS9"]
