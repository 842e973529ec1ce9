"""The part of a WannierTools input file (wt.in) that the surface-state path reads,
and the surface geometry the reference derives from it.

Reading (src/readinput.f90):

* namelists &TB_FILE (Hrfile), &CONTROL (SlabSS_calc, SlabArc_calc), &SYSTEM (SOC,
  E_FERMI) and &PARAMETERS (Eta_Arc / Fermi_broadening, E_arc / iso_energy,
  OmegaNum, OmegaMin, OmegaMax, Nk1, Nk2, NP), with the reference's defaults
  (:586-597) and the legacy Eta_Arc / E_arc overrides (:664-666); energies stay
  in eV here and are converted where they are used (:721-724);
* cards LATTICE (:760-790; Angstrom or Bohr), ATOM_POSITIONS (:849-930; Direct or
  Cartesian), PROJECTORS (:996-1085; orbitals per atom, the spin-down copy of
  every orbital after all spin-up ones when SOC > 0), SURFACE (:1576-1630; two
  or three rows of Umatrix, the third (0, 0, 1) when absent or unreadable),
  KPATH_SLAB (:2134-2213), KPLANE_SLAB (:2217-2262) and SURFACE_ATOMS
  (:2851-2955; atom index lists with ranges, default every atom).

A card is found, as the reference does, by the first token of a line (upper
cased); numbers are read list-directed: the first tokens of the following
lines, a 'd' exponent read as 'e', the rest of a line (comments) ignored.

Geometry (src/readinput.f90:1632-1870): the cell volume check of the SURFACE
vectors and, when it fails, the search for a third lattice vector of the same
volume (FindTheThirdLatticeVector, :4247-4463); the atom positions in the
surface cell (rotate_newlattice, transformtohomecell, then the shift that puts
the topmost atom at 0.95 along R3'); the frame Urot (x along R1', z along
R1' x R2'); the 2D lattice Ra2, Rb2 and reciprocal Ka2, Kb2; the k-path
lengths k2len (:2180-2200) and the k plane in Cartesian units
(src/fermiarc.f90:140-150).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

ANGSTROM2ATOMIC = 1.0 / 0.529177210903   # src/module.f90:711
PI_REF = 3.14159265358979                # src/module.f90:719
EPS9 = float(np.float32(1e-9))           # src/module.f90:728 (single-precision literal)


@dataclass
class WtInput:
    """The surface-state subset of a wt.in (energies in eV, lengths in Bohr)."""
    hrfile: str = "wannier90_hr.dat"
    slab_ss: bool = False
    slab_arc: bool = False
    soc: int = 0
    e_fermi: float = 0.0
    omeganum: int = 100
    omegamin: float = -1.0
    omegamax: float = 1.0
    fermi_broadening: float = 0.005
    iso_energy: float = 0.0
    nk1: int = 10
    nk2: int = 10
    np_: int = 2
    lattice: np.ndarray = field(default_factory=lambda: np.eye(3))       # rows a1, a2, a3 (Bohr)
    atom_names: list = field(default_factory=list)
    pos_direct: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    nprojs: list = field(default_factory=list)
    umatrix: np.ndarray = field(default_factory=lambda: np.eye(3))
    surface_card: bool = False
    kpath_lines: list = field(default_factory=list)   # [(name, kstart(2), name, kend(2))]
    kplane: tuple = ((-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    top_atoms: list | None = None                     # 1-based; None = every atom
    bottom_atoms: list | None = None

    @property
    def num_wann(self) -> int:
        n = sum(self.nprojs)
        return 2 * n if self.soc > 0 else n


def _num(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "E"))


def _tokens(line: str) -> list[str]:
    return [t for t in re.split(r"[\s,]+", line.strip()) if t]


def _expand(tokens: list[str]) -> list[str]:
    """List-directed repeat counts: 'r*c' stands for r copies of c."""
    out = []
    for t in tokens:
        m = re.fullmatch(r"(\d+)\*(.+)", t)
        out.extend([m.group(2)] * int(m.group(1)) if m else [t])
    return out


def _namelists(text: str) -> dict[str, dict[str, str]]:
    """&NAME key = value, ... / blocks: {NAME: {KEY: raw value}} (comments after '!')."""
    out: dict[str, dict[str, str]] = {}
    for m in re.finditer(r"&(\w+)(.*?)(?:^\s*/\s*$|/\s*$)", text, flags=re.S | re.M):
        name = m.group(1).upper()
        body = "\n".join(line.split("!", 1)[0] for line in m.group(2).splitlines())
        vals: dict[str, str] = {}
        for km in re.finditer(r"(\w+)\s*=\s*('[^']*'|\"[^\"]*\"|[^,\n=]+?)(?=\s*(?:,|\n|$|\w+\s*=))",
                              body):
            vals[km.group(1).upper()] = km.group(2).strip()
        out[name] = vals
    return out


def _logical(v: str) -> bool:
    v = v.strip().strip(".").upper()
    return v.startswith("T")


def _card(lines: list[str], name: str) -> int | None:
    """Index of the line after the card's keyword line, or None."""
    for i, line in enumerate(lines):
        t = _tokens(line)
        if t and t[0].upper() == name:
            return i + 1
    return None


def _values(lines: list[str], i: int, n: int, skip_blank: bool = True):
    """The first n numbers of the next line from i on (list-directed read of n
    reals: blank lines skipped); (values, next index), or (None, i) if the line
    does not start with n numbers."""
    while skip_blank and i < len(lines) and not _tokens(lines[i]):
        i += 1
    if i >= len(lines):
        return None, i
    t = _expand(_tokens(lines[i]))
    try:
        return [_num(x) for x in t[:n]] if len(t) >= n else None, i + 1
    except ValueError:
        return None, i


def _ranges(line: str) -> list[int]:
    """An index list with ranges ('1 3-5 8' -> 1 3 4 5 8), as param_get_range_vector."""
    out = []
    for t in _tokens(line.split("!", 1)[0]):
        if "-" in t[1:]:
            a, b = t.split("-", 1)
            out.extend(range(int(a), int(b) + 1))
        else:
            out.append(int(t))
    return out


def read_wt_in(path) -> WtInput:
    text = Path(path).read_text()
    lines = text.splitlines()
    nl = _namelists(text)
    w = WtInput()
    tb = nl.get("TB_FILE", {})
    if "HRFILE" in tb:
        w.hrfile = tb["HRFILE"].strip("'\"")
    ctl = nl.get("CONTROL", {})
    w.slab_ss = _logical(ctl.get("SLABSS_CALC", "F"))
    w.slab_arc = _logical(ctl.get("SLABARC_CALC", "F"))
    sy = nl.get("SYSTEM", {})
    w.soc = int(_num(sy.get("SOC", "0")))
    w.e_fermi = _num(sy.get("E_FERMI", "0"))
    par = nl.get("PARAMETERS", {})
    w.omeganum = int(_num(par.get("OMEGANUM", "100")))
    w.omegamin = _num(par.get("OMEGAMIN", "-1"))
    w.omegamax = _num(par.get("OMEGAMAX", "1"))
    w.fermi_broadening = _num(par.get("FERMI_BROADENING", "0.005"))
    w.iso_energy = _num(par.get("ISO_ENERGY", "0"))
    eta_arc = _num(par.get("ETA_ARC", "-999"))
    e_arc = _num(par.get("E_ARC", "-999"))
    if eta_arc > -998.0:                                   # src/readinput.f90:665-666
        w.fermi_broadening = eta_arc
    if e_arc > -998.0:
        w.iso_energy = e_arc
    w.nk1 = int(_num(par.get("NK1", "10")))
    w.nk2 = int(_num(par.get("NK2", "10")))
    w.np_ = int(_num(par.get("NP", "2")))

    i = _card(lines, "LATTICE")
    if i is None:
        raise ValueError("wt.in: no LATTICE card")
    unit = _tokens(lines[i])[0].upper()
    lat = []
    i += 1
    for _ in range(3):
        v, i = _values(lines, i, 3)
        if v is None:
            raise ValueError("wt.in: bad LATTICE vector")
        lat.append(v)
    w.lattice = np.array(lat, float) * (ANGSTROM2ATOMIC if "ANG" in unit else 1.0)

    i = _card(lines, "ATOM_POSITIONS")
    if i is None:
        raise ValueError("wt.in: no ATOM_POSITIONS card")
    v, i = _values(lines, i, 1)
    nat = int(v[0])
    while not _tokens(lines[i]):
        i += 1
    direct = "D" in _tokens(lines[i])[0]                   # index(DirectOrCart, "D") > 0
    i += 1
    pos = []
    for _ in range(nat):
        while not _tokens(lines[i]):
            i += 1
        t = _tokens(lines[i])
        w.atom_names.append(t[0])
        p = np.array([_num(x) for x in t[1:4]])
        if direct:
            pos.append(p)
        else:
            cart = p * (ANGSTROM2ATOMIC if "ANG" in unit else 1.0)
            pos.append(np.linalg.solve(w.lattice.T, cart))
        i += 1
    w.pos_direct = np.array(pos, float).reshape(nat, 3)

    i = _card(lines, "PROJECTORS")
    if i is None:
        i = _card(lines, "PROJECTOR")
    if i is None:
        raise ValueError("wt.in: no PROJECTORS card")
    while not _tokens(lines[i]):
        i += 1
    counts = []
    while len(counts) < nat:                               # read(1001, *) nprojs: may span lines
        counts.extend(int(x) for x in _expand(_tokens(lines[i].split("!", 1)[0])))
        i += 1
    w.nprojs = counts[:nat]

    i = _card(lines, "SURFACE")
    if i is not None:
        w.surface_card = True
        u1, i = _values(lines, i, 3)
        u2, i = _values(lines, i, 3)
        u3, _ = _values(lines, i, 3)                       # unreadable third row: (0, 0, 1)
        if u1 is None or u2 is None:
            raise ValueError("wt.in: bad SURFACE card")
        w.umatrix = np.array([u1, u2, u3 if u3 is not None else [0.0, 0.0, 1.0]], float)

    i = _card(lines, "KPATH_SLAB")
    if i is not None:
        v, i = _values(lines, i, 1)
        for _ in range(int(v[0])):
            while not _tokens(lines[i]):
                i += 1
            t = _tokens(lines[i])
            w.kpath_lines.append((t[0], (_num(t[1]), _num(t[2])), t[3], (_num(t[4]), _num(t[5]))))
            i += 1

    i = _card(lines, "KPLANE_SLAB")
    if i is not None:
        s, i = _values(lines, i, 2)
        a, i = _values(lines, i, 2)
        b, i = _values(lines, i, 2)
        if s is None or a is None or b is None:
            raise ValueError("wt.in: KPLANE_SLAB needs a start point and two vectors")
        w.kplane = (tuple(s), tuple(a), tuple(b))

    i = _card(lines, "SURFACE_ATOMS")
    if i is not None:
        w.top_atoms = _ranges(lines[i])
        w.bottom_atoms = _ranges(lines[i + 1])
    return w


def orbital_atoms(nprojs, soc: int) -> np.ndarray:
    """0-based atom of each (spin) orbital: the orbitals of atom 1, then atom 2, ...;
    with SOC the same order again for spin down (src/readinput.f90:1066-1085)."""
    a = np.concatenate([np.full(n, ia, np.int64) for ia, n in enumerate(nprojs)]) if nprojs else \
        np.zeros(0, np.int64)
    return np.concatenate([a, a]) if soc > 0 else a


def surface_orbitals(w: WtInput):
    """TopOrbitals, BottomOrbitals (1-based) of the SURFACE_ATOMS lists
    (src/readinput.f90:2915-2950)."""
    nat = len(w.nprojs)
    start = np.concatenate([[1], 1 + np.cumsum(w.nprojs)[:-1]]) if nat else np.zeros(0, int)
    half = sum(w.nprojs)

    def orbs(atoms):
        atoms = atoms if atoms is not None else list(range(1, nat + 1))
        up = [int(start[a - 1]) + j for a in atoms for j in range(w.nprojs[a - 1])]
        return up + ([o + half for o in up] if w.soc > 0 else [])
    return orbs(w.top_atoms), orbs(w.bottom_atoms)


def _third_vector(u: np.ndarray, lat: np.ndarray, irmax: int = 6) -> np.ndarray:
    """FindTheThirdLatticeVector (src/readinput.f90:4247-4463): each of the first two
    rows becomes the shortest lattice vector parallel to it (same direction), and
    the third the shortest one, in the search's loop order, that spans the
    smallest non-zero volume with them; sign chosen for a right-handed cell."""
    u = u.copy()
    rng = range(-irmax, irmax + 1)
    cand = [(i1, i2, i3) for i1 in rng for i2 in rng for i3 in rng if (i1, i2, i3) != (0, 0, 0)]
    for row in (0, 1):
        best, blen = None, 9999999.0
        for c in cand:
            cr = np.cross(u[row], c)
            if np.abs(cr).sum() < EPS9 and np.dot(u[row], c) > 0:
                ln = np.linalg.norm(np.array(c) @ lat)
                if ln < blen:
                    best, blen = c, ln
        if best is not None:
            u[row] = best
    r1, r2 = u[0] @ lat, u[1] @ lat
    vols = [abs(np.dot(r1, np.cross(r2, np.array(c) @ lat))) for c in cand]
    vmin = min(v for v in vols if v >= EPS9)
    lmin = min(np.linalg.norm(np.array(c) @ lat) for c, v in zip(cand, vols) if abs(v - vmin) < EPS9)
    for c, v in zip(cand, vols):
        if abs(v - vmin) < EPS9 and abs(np.linalg.norm(np.array(c) @ lat) - lmin) < EPS9:
            u[2] = c
            break
    if np.dot(r1, np.cross(r2, u[2] @ lat)) < 0:
        u[2] = -u[2]
    return u


def _home(p: np.ndarray) -> np.ndarray:
    """transformtohomecell (src/readinput.f90:4495-4520): each coordinate into [0, 1)."""
    p = p.copy()
    for i in range(3):
        while not (0.0 <= p[i] < 1.0):
            p[i] += 1.0 if p[i] < 0.0 else -1.0
    return p


@dataclass
class SurfaceGeometry:
    umatrix: np.ndarray          # rows: R1', R2', R3' in units of a1, a2, a3
    cell: np.ndarray             # rows R1', R2', R3' (Cartesian, Bohr)
    pos_new: np.ndarray          # atoms in the surface cell, direct (after the top-surface shift)
    urot: np.ndarray             # rows e_x', e_y', e_z'
    ka2: np.ndarray
    kb2: np.ndarray


def surface_geometry(w: WtInput) -> SurfaceGeometry:
    lat = w.lattice
    u = w.umatrix.astype(float).copy()
    vol0 = abs(np.dot(lat[0], np.cross(lat[1], lat[2])))
    vol = np.dot(u[0] @ lat, np.cross(u[1] @ lat, u[2] @ lat))
    if vol < 0:                                             # :1645-1648
        u[2] = -u[2]
    if abs(abs(vol) - vol0) > 0.001:                        # :1658-1660
        u = _third_vector(u, lat)
    cell = u @ lat
    uinv = np.linalg.inv(u)
    pos = np.array([_home(uinv.T @ p) for p in w.pos_direct])       # rotate_newlattice + home
    if len(pos):
        top = int(np.argmax(pos[:, 2]))                     # the first atom of largest R3' coordinate
        shift = np.array([0.0, 0.0, 0.95 - pos[top, 2]])
        pos = np.array([_home(p + shift) for p in pos])
    r1, r2 = cell[0], cell[1]
    ex = r1 / np.linalg.norm(r1)
    ez = np.cross(r1, r2)
    ez = ez / np.linalg.norm(ez)
    ey = np.cross(ez, ex)
    ey = ey / np.linalg.norm(ey)
    urot = np.array([ex, ey, ez])
    ra2 = np.array([urot[0] @ r1, urot[1] @ r1])
    rb2 = np.array([urot[0] @ r2, urot[1] @ r2])
    area = abs(ra2[0] * rb2[1] - rb2[0] * ra2[1])
    if area < 1e-6:
        raise ValueError("surface cell has zero area")
    ka2 = np.array([2.0 * PI_REF / area * rb2[1], -2.0 * PI_REF / area * rb2[0]])
    kb2 = np.array([-2.0 * PI_REF / area * ra2[1], 2.0 * PI_REF / area * ra2[0]])
    return SurfaceGeometry(u, cell, pos, urot, ka2, kb2)


def kpath(w: WtInput, geo: SurfaceGeometry):
    """k2_path (knv2, 2) in fractions of Ka2, Kb2 and k2len (knv2) in 1/Bohr:
    Nk1 points per line, endpoints included (src/readinput.f90:2180-2200)."""
    nn = w.nk1
    kp = np.zeros((nn * len(w.kpath_lines), 2))
    klen = np.zeros(nn * len(w.kpath_lines))
    t1 = 0.0
    for j, (_, ks, _, ke) in enumerate(w.kpath_lines):
        ks, ke = np.asarray(ks, float), np.asarray(ke, float)
        k1 = ks[0] * geo.ka2 + ks[1] * geo.kb2
        k2 = ke[0] * geo.ka2 + ke[1] * geo.kb2
        step = np.sqrt((k2[0] - k1[0]) ** 2 + (k2[1] - k1[1]) ** 2) / float(nn - 1)
        for i in range(1, nn + 1):
            kp[i - 1 + j * nn] = ks + (ke - ks) * (i - 1) / float(nn - 1)
            if i > 1:
                t1 += step
            klen[i - 1 + j * nn] = t1
    return kp, klen


def kplane(w: WtInput, geo: SurfaceGeometry):
    """(nkx, nky, k12 (nkx nky, 2) fractional, k12_shape Cartesian 1/Bohr): SurfaceDOSkk's
    plane, Nk1 / Nk2 bumped to odd, second index fastest (src/fermiarc.f90:68-70,140-150)."""
    from .api import kplane_slab
    nkx, nky, k12 = kplane_slab(w.nk1, w.nk2, *w.kplane)
    shape = k12[:, :1] * geo.ka2[None, :] + k12[:, 1:2] * geo.kb2[None, :]
    return nkx, nky, k12, shape
