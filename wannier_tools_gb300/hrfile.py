"""wannier90_hr.dat input and the surface-cell remap, host side.

* ``read_hr``         readNormalHmnR's dense branch, src/readHmnR.f90:43-160:
                      comment line, num_wann, nrpts, the ndegen list (15 per
                      line), then "R1 R2 R3 m n Re Im" lines; R vectors are
                      deduplicated in order of first appearance
                      (src/readHmnR.f90:100-125).
* ``to_hartree``      E_fermi removed from the R = 0 diagonal and eV -> Hartree
                      (src/readHmnR.f90:141-159).
* ``get_hmnr_cell``   the surface-cell remap of src/readHmnR.f90:578-766 for any
                      SURFACE card: each hopping H_ij(R) moves to
                      R' = U^-T (R + tau_j - tau_i) - (tau'_j - tau'_i), rounded
                      half away from zero (ANINT), the orbitals' atoms at tau in
                      the original cell and tau' in the surface cell; R' with a
                      component beyond 8 is dropped; R' ordered R1 fastest then
                      R2 then R3; values divided by ndegen, which becomes 1; a
                      later (R, i, j) mapped to the same (R', i, j) replaces an
                      earlier one, as the reference's assignment does.
* ``surface_cell``    the same for a SURFACE card that keeps the lattice and
                      every orbital at the origin (R' = R).
* ``write_hr``        the wannier90_hr.dat text layout (as written for
                      wannier90_hr_newcell.dat, src/readHmnR.f90:738-758).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

EV2HARTREE = 1.0 / 27.211385          # src/module.f90:713
MAX_IR = 8                            # src/readHmnR.f90:606


def read_hr(path) -> dict:
    """Parse a dense wannier90_hr.dat; energies stay in eV."""
    lines = Path(path).read_text().splitlines()
    pos = 1                                   # skip the comment line
    nw = int(lines[pos].split()[0])
    pos += 1
    if nw <= 0:
        raise ValueError("num_wann is zero in hr file")
    nrpts = int(lines[pos].split()[0])
    pos += 1
    ndegen: list[int] = []
    while len(ndegen) < nrpts:
        ndegen.extend(int(x) for x in lines[pos].split())
        pos += 1
    irvec = np.zeros((nrpts, 3), dtype=np.int32)
    hmnr = np.zeros((nrpts, nw, nw), dtype=np.complex128)
    index: dict[tuple[int, int, int], int] = {}
    for line in lines[pos:]:
        parts = line.split()
        if len(parts) < 7:
            continue
        r = (int(parts[0]), int(parts[1]), int(parts[2]))
        m, n = int(parts[3]), int(parts[4])
        idx = index.get(r)
        if idx is None:
            idx = len(index)
            if idx >= nrpts:
                raise ValueError("more distinct R vectors than nrpts")
            index[r] = idx
            irvec[idx] = r
        hmnr[idx, m - 1, n - 1] = complex(float(parts[5]), float(parts[6]))
    return {"nw": nw, "nrpts": nrpts, "irvec": irvec, "ndegen": np.asarray(ndegen[:nrpts], np.int32),
            "hmnr": hmnr}


def to_hartree(hr: dict, e_fermi_ev: float = 0.0) -> dict:
    out = dict(hr)
    h = hr["hmnr"].copy()
    for r in range(h.shape[0]):
        if tuple(hr["irvec"][r]) == (0, 0, 0):
            h[r][np.diag_indices(h.shape[1])] -= e_fermi_ev
    out["hmnr"] = h * EV2HARTREE
    return out


def _anint(x: np.ndarray) -> np.ndarray:
    """Fortran ANINT: nearest integer, halves away from zero."""
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def get_hmnr_cell(hr: dict, umatrix, orb_atom, pos_old, pos_new, max_ir: int = MAX_IR) -> dict:
    """HmnR of the cell defined by the SURFACE card (see module docstring).

    hr        irvec (nR, 3), ndegen (nR,), hmnr (nR, nw, nw)
    umatrix   3 x 3, rows R1', R2', R3' in units of the original lattice vectors
    orb_atom  (nw,) 0-based atom of each orbital (the same in both cells)
    pos_old   (natoms, 3) direct coordinates in the original cell
    pos_new   (natoms, 3) direct coordinates in the surface cell
    """
    irv = np.asarray(hr["irvec"], dtype=np.float64)
    h = np.asarray(hr["hmnr"])
    nd = np.asarray(hr["ndegen"], dtype=np.float64)
    nR, nw, _ = h.shape
    uinv_t = np.linalg.inv(np.asarray(umatrix, dtype=np.float64)).T
    ta = np.asarray(pos_old, dtype=np.float64)[np.asarray(orb_atom)]       # (nw, 3)
    tb = np.asarray(pos_new, dtype=np.float64)[np.asarray(orb_atom)]
    dold = ta[None, :, :] - ta[:, None, :]          # [i, j] = tau_j - tau_i
    dnew = tb[None, :, :] - tb[:, None, :]
    rnew = np.empty((nR, nw, nw, 3), dtype=np.int64)
    for r in range(nR):
        rmn = irv[r][None, None, :] + dold
        rnew[r] = _anint(rmn @ uinv_t.T - dnew).astype(np.int64)
    keep = np.all(np.abs(rnew) <= max_ir, axis=-1)
    present = np.unique(rnew[keep].reshape(-1, 3), axis=0)
    order = present[np.lexsort((present[:, 0], present[:, 1], present[:, 2]))]
    span = 2 * max_ir + 1
    key = lambda v: ((v[..., 2] + max_ir) * span + (v[..., 1] + max_ir)) * span + (v[..., 0] + max_ir)
    slot = np.full(span ** 3, -1, dtype=np.int64)
    slot[key(order)] = np.arange(len(order))
    out = np.zeros((len(order), nw, nw), dtype=np.complex128)
    ii, jj = np.meshgrid(np.arange(nw), np.arange(nw), indexing="ij")
    for r in range(nR):                              # in R order: later entries replace earlier
        k = keep[r]
        out[slot[key(rnew[r][k])], ii[k], jj[k]] = h[r][k] / nd[r]
    return {"nw": nw, "irvec": order.astype(np.int32).reshape(-1, 3),
            "ndegen": np.ones(len(order), np.int32), "hmnr": out}


def surface_cell(hr: dict) -> dict:
    """Surface-cell arrays for an identity Umatrix (see module docstring)."""
    irv = hr["irvec"]
    keep = np.all(np.abs(irv) <= MAX_IR, axis=1)
    present = {tuple(v) for v in irv[keep]}
    order = sorted(present, key=lambda v: (v[2], v[1], v[0]))
    slot = {v: i for i, v in enumerate(order)}
    nw = hr["hmnr"].shape[1]
    h = np.zeros((len(order), nw, nw), dtype=np.complex128)
    for r in range(irv.shape[0]):
        v = tuple(irv[r])
        if v in slot:
            h[slot[v]] = hr["hmnr"][r] / float(hr["ndegen"][r])
    return {"nw": nw, "irvec": np.array(order, dtype=np.int32).reshape(-1, 3),
            "ndegen": np.ones(len(order), np.int32), "hmnr": h}


def write_hr(path, irvec, ndegen, hmnr_ev, header: str = "written by wannier_tools_gb300") -> None:
    nR, nw, _ = hmnr_ev.shape
    out = [header, f"{nw:12d}", f"{nR:12d}"]
    for s in range(0, nR, 15):
        out.append("".join(f"{int(d):5d}" for d in ndegen[s:s + 15]))
    for r in range(nR):
        for j in range(nw):
            for i in range(nw):
                v = hmnr_ev[r, i, j]
                out.append(f"{irvec[r, 0]:5d}{irvec[r, 1]:5d}{irvec[r, 2]:5d}{i + 1:5d}{j + 1:5d}"
                           f"{v.real:16.8f}{v.imag:16.8f}")
    Path(path).write_text("\n".join(out) + "\n")
