"""The reference's surface-state calculations as a drop-in: a wt.in and its
wannier90_hr.dat in, the reference's output files out, every (k, omega)
decimation on the GPU.

``run(wt_in)`` follows the two branches of the reference's main program that
this path serves (src/main.f90:714-735):

* the model: the hr file named in &TB_FILE read as readNormalHmnR does
  (E_FERMI removed, eV -> Hartree; src/readHmnR.f90:43-160) and remapped into
  the cell of the SURFACE card (get_hmnr_cell, src/readHmnR.f90:578-766), with
  the surface geometry, orbital lists and k grids of src/readinput.f90
  (``wtin``);
* SlabSS_calc -> surfstat (src/surfstat.f90:1-320): the KPATH_SLAB path of Nk1
  points per line, OmegaNum energies from OmegaMin (OmegaMax excluded) at
  eta = 3 (OmegaMax - OmegaMin) / OmegaNum; dos.dat_l / dos.dat_r / dos.dat_bulk
  and spindos.dat_l / spindos.dat_r (spin sums rotated into the SURFACE frame);
* SlabArc_calc -> SurfaceDOSkk (src/fermiarc.f90:1-460): the KPLANE_SLAB plane
  at E_arc with Eta_Arc broadening; arc.dat_l / arc.dat_r / arc.dat_bulk.

Command line: ``python -m wannier_tools_gb300.dropin wt.in [outdir] [--mixed]``.
"""
from __future__ import annotations

import argparse
from pathlib import Path

import numpy as np

from . import hrfile, outfiles, wtin
from .api import ACCURACY_REF, EV2HARTREE, ITERMAX_REF, PREC_FP64, PREC_MIXED, Model, surfstat_grid


def load_model(wt_in_path, hr_path=None):
    """(input, geometry, surface-cell model arrays, TopOrbitals, BottomOrbitals)."""
    path = Path(wt_in_path)
    w = wtin.read_wt_in(path)
    geo = wtin.surface_geometry(w)
    hr = hrfile.read_hr(Path(hr_path) if hr_path else path.parent / w.hrfile)
    if hr["nw"] != w.num_wann:
        raise ValueError(f"hr file has {hr['nw']} orbitals, the PROJECTORS card {w.num_wann}")
    hr = hrfile.to_hartree(hr, w.e_fermi)
    cell = hrfile.get_hmnr_cell(hr, geo.umatrix, wtin.orbital_atoms(w.nprojs, w.soc), w.pos_direct,
                                geo.pos_new)
    top, bot = wtin.surface_orbitals(w)
    return w, geo, cell, top, bot


def run(wt_in_path, outdir=None, precision: int = PREC_FP64, hr_path=None,
        tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF) -> dict:
    """Run the wt.in's SlabSS / SlabArc calculations; write their files to outdir
    (the wt.in's directory by default).  Returns the raw results and the paths."""
    w, geo, cell, top, bot = load_model(wt_in_path, hr_path)
    out = Path(outdir) if outdir is not None else Path(wt_in_path).parent
    res: dict = {"input": w, "geometry": geo, "files": []}
    with Model(cell["hmnr"], cell["irvec"], cell["ndegen"], w.np_) as model:
        if w.slab_ss:
            kp, klen = wtin.kpath(w, geo)
            omega, eta = surfstat_grid(w.omegamin * EV2HARTREE, w.omegamax * EV2HARTREE, w.omeganum)
            r = model.surface_spectrum_spin(kp, omega, eta, top, bot, arc=False, tol=tol, itermax=itermax,
                                            precision=precision)
            spin = {k: r[k] for k in ("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r")}
            res["files"] += outfiles.write_surfstat(out, klen, omega, r["dos_l"], r["dos_r"],
                                                    r["dos_bulk"], spin=spin, rotation=geo.urot)
            res["surfstat"] = dict(r, k2_path=kp, k2len=klen, omega=omega, eta=eta)
        if w.slab_arc:
            nkx, nky, k12, shape = wtin.kplane(w, geo)
            r = model.surface_spectrum(k12, [w.iso_energy * EV2HARTREE], w.fermi_broadening * EV2HARTREE,
                                       top, bot, tol=tol, itermax=itermax, divide_by_pi=True,
                                       precision=precision)
            res["files"] += outfiles.write_arc(out, shape, r["dos_l"][:, 0], r["dos_r"][:, 0],
                                               r["dos_bulk"][:, 0], nky)
            res["arc"] = dict(r, k12=k12, k12_shape=shape, nkx=nkx, nky=nky)
    return res


def read_dat(path) -> np.ndarray:
    """The numbers of one of the written .dat files, one row per record (comment
    and blank records skipped)."""
    rows = []
    for line in Path(path).read_text().splitlines():
        s = line.strip()
        if not s or s.startswith("#"):
            continue
        rows.append([float(x) for x in s.split()])
    return np.array(rows)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("wt_in")
    ap.add_argument("outdir", nargs="?", default=None)
    ap.add_argument("--mixed", action="store_true", help="split-BF16 tensor-core form (1e-5)")
    a = ap.parse_args(argv)
    from . import build
    build()
    res = run(a.wt_in, a.outdir, PREC_MIXED if a.mixed else PREC_FP64)
    for f in res["files"]:
        print(f)


if __name__ == "__main__":
    main()
