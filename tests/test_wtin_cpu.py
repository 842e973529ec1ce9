"""wt.in reading, the surface geometry and the general surface-cell remap (no GPU).

The reader is run on the reference's own Weyl example input (copied into
tests/golden) and on inputs written here that use the forms the reader
handles (Cartesian positions, three-row SURFACE cards, several k lines,
SURFACE_ATOMS ranges, repeat counts).  get_hmnr_cell is compared with the
oracle's step-by-step restatement of src/readHmnR.f90:578-766 on the Weyl
model and on multi-atom models with non-trivial SURFACE cards."""
import numpy as np
import pytest

from oracle import wt_oracle as O
from wannier_tools_gb300 import hrfile, wtin

from .conftest import GOLDEN

A2B = wtin.ANGSTROM2ATOMIC


def test_weyl_example_input():
    w = wtin.read_wt_in(GOLDEN / "weyl3d_wt.in")
    assert w.hrfile == "Weyl3D_hr.dat" and w.slab_ss and w.slab_arc and w.soc == 1
    assert (w.omeganum, w.omegamin, w.omegamax) == (400, -1.6, 1.6)
    assert w.fermi_broadening == 0.001 and w.iso_energy == 0.0          # Eta_Arc, E_arc
    assert (w.nk1, w.nk2, w.np_) == (201, 201, 2)
    assert np.allclose(w.lattice, np.eye(3) * A2B)
    assert w.atom_names == ["A"] and np.allclose(w.pos_direct, 0) and w.nprojs == [1]
    assert w.num_wann == 2
    # two SURFACE rows; the third line is KPATH_SLAB, so the third row stays (0, 0, 1)
    assert np.allclose(w.umatrix, [[1, 0, 0], [0, 0, 1], [0, 0, 1]])
    assert w.kpath_lines == [("-X", (-0.5, 0.0), "X", (0.5, 0.0))]
    assert w.kplane == ((-0.5, -0.5), (1.0, 0.0), (0.0, 1.0))
    top, bot = wtin.surface_orbitals(w)
    assert top == [1, 2] and bot == [1, 2]                              # both spins of atom 1
    g = wtin.surface_geometry(w)
    # the volume check fails (R2' = R3'), so the third vector is searched: (0, -1, 0)
    assert np.allclose(g.umatrix, [[1, 0, 0], [0, 0, 1], [0, -1, 0]])
    assert np.allclose(g.pos_new, [[0, 0, 0.95]])                      # top atom at 0.95
    assert np.allclose(g.urot, [[1, 0, 0], [0, 0, 1], [0, -1, 0]])
    assert np.allclose(g.ka2, [2 * wtin.PI_REF / A2B, 0]) and np.allclose(g.kb2, [0, 2 * wtin.PI_REF / A2B])
    kp, klen = wtin.kpath(w, g)
    assert kp.shape == (201, 2) and np.allclose(kp[[0, 100, 200]], [[-0.5, 0], [0, 0], [0.5, 0]])
    assert np.isclose(klen[-1] * A2B, 2 * wtin.PI_REF)                 # |Ka2| in 1/Angstrom


WT_IN = """&TB_FILE
Hrfile = 'model_hr.dat'
/
&CONTROL
SlabSS_calc = .true., SlabArc_calc = F
/
&SYSTEM
SOC = 0, E_FERMI = 0.25d0   ! shift
/
&PARAMETERS
Fermi_broadening = 2d-3
iso_energy = 0.1
OmegaNum = 12, OmegaMin = -0.5
OmegaMax = 0.5
Nk1 = 7
Nk2 = 6
NP = 3
/

LATTICE
Angstrom
   3.0   0.0   0.0
   0.5   2.8   0.0   ! a tilted one
   0.0   0.0   5.0

ATOM_POSITIONS
3
Cartesian
A   0.00  0.00  0.00
B   1.75  1.40  1.25
C   0.50  2.80  3.50

PROJECTORS
 2*2 1
A s pz
B s px
C s

SURFACE
 1  1  0
 0  0  1
 1  0  0

KPATH_SLAB
2
G 0.0 0.0 X 0.5 0.0
X 0.5 0.0 M 0.5 0.5

KPLANE_SLAB
-0.25 -0.25
 0.5  0.0
 0.0  0.5

SURFACE_ATOMS
1-2
3 1
"""


def test_synthetic_input_forms(tmp_path):
    p = tmp_path / "wt.in"
    p.write_text(WT_IN)
    w = wtin.read_wt_in(p)
    assert w.hrfile == "model_hr.dat" and w.slab_ss and not w.slab_arc
    assert w.soc == 0 and w.e_fermi == 0.25 and w.fermi_broadening == 2e-3 and w.iso_energy == 0.1
    assert (w.nk1, w.nk2, w.np_) == (7, 6, 3)
    assert w.nprojs == [2, 2, 1] and w.num_wann == 5
    lat = np.array([[3, 0, 0], [0.5, 2.8, 0], [0, 0, 5]]) * A2B
    assert np.allclose(w.lattice, lat)
    # Cartesian positions back to direct coordinates
    assert np.allclose(w.pos_direct @ lat, np.array([[0, 0, 0], [1.75, 1.4, 1.25], [0.5, 2.8, 3.5]]) * A2B)
    assert np.allclose(w.umatrix, [[1, 1, 0], [0, 0, 1], [1, 0, 0]])
    assert w.top_atoms == [1, 2] and w.bottom_atoms == [3, 1]
    assert wtin.surface_orbitals(w) == ([1, 2, 3, 4], [5, 1, 2])
    assert list(wtin.orbital_atoms(w.nprojs, w.soc)) == [0, 0, 1, 1, 2]
    g = wtin.surface_geometry(w)
    # a right-handed cell of the original volume
    cell = g.umatrix @ lat
    assert np.isclose(np.dot(cell[0], np.cross(cell[1], cell[2])), abs(np.linalg.det(lat)))
    assert np.all((g.pos_new >= 0) & (g.pos_new < 1)) and np.isclose(g.pos_new[:, 2].max(), 0.95)
    # Ka2, Kb2 are the reciprocal basis of the 2D cell in the rotated frame
    r2 = np.array([[g.urot[0] @ cell[0], g.urot[1] @ cell[0]], [g.urot[0] @ cell[1], g.urot[1] @ cell[1]]])
    kk = np.array([g.ka2, g.kb2])
    assert np.allclose(r2 @ kk.T, 2 * wtin.PI_REF * np.eye(2))
    kp, klen = wtin.kpath(w, g)
    assert kp.shape == (14, 2) and np.allclose(kp[6], [0.5, 0]) and np.allclose(kp[7], [0.5, 0])
    assert klen[7] == klen[6] and np.isclose(klen[6], np.linalg.norm(0.5 * g.ka2))   # lines join
    nkx, nky, k12, shape = wtin.kplane(w, g)
    assert (nkx, nky) == (7, 7) and np.allclose(k12[0], [-0.25, -0.25]) and np.allclose(k12[-1], [0.25, 0.25])


@pytest.mark.parametrize("surface", [
    [[1, 0, 0], [0, 0, 1], [0, 0, 1]],      # third row unreadable: searched
    [[0, 1, 0], [0, 0, 1], [1, 0, 0]],
    [[1, 1, 0], [0, 0, 1], [0, 1, 0]],      # left-handed as given: the third row flips
    [[1, -1, 0], [1, 1, 1], [0, 0, 1]],     # a larger cell: searched
])
def test_third_vector_keeps_the_volume(surface):
    w = wtin.WtInput()
    w.lattice = np.array([[2.0, 0.0, 0.0], [0.7, 1.9, 0.0], [0.3, 0.4, 3.1]])
    w.pos_direct = np.array([[0.1, 0.2, 0.3]])
    w.nprojs = [1]
    w.umatrix = np.array(surface, float)
    g = wtin.surface_geometry(w)
    cell = g.umatrix @ w.lattice
    vol = np.dot(cell[0], np.cross(cell[1], cell[2]))
    assert np.isclose(vol, abs(np.linalg.det(w.lattice)))
    assert np.allclose(g.umatrix, np.round(g.umatrix))          # integer combinations
    assert np.isclose(abs(np.linalg.det(g.umatrix)), 1.0)


def _random_hr(nw, rmax, seed):
    rng = np.random.default_rng(seed)
    rs = [(a, b, c) for c in range(-rmax, rmax + 1) for b in range(-rmax, rmax + 1)
          for a in range(-rmax, rmax + 1)]
    rng.shuffle(rs)
    irv = np.array(rs, np.int32)
    h = rng.normal(size=(len(rs), nw, nw)) + 1j * rng.normal(size=(len(rs), nw, nw))
    nd = rng.integers(1, 4, len(rs)).astype(np.int32)
    return {"nw": nw, "irvec": irv, "ndegen": nd, "hmnr": h}


def test_remap_weyl_example_matches_oracle():
    w = wtin.read_wt_in(GOLDEN / "weyl3d_wt.in")
    g = wtin.surface_geometry(w)
    d = np.load(GOLDEN / "weyl3d_hr_model.npz")
    hr = hrfile.to_hartree({"nw": 2, "irvec": d["irvec"], "ndegen": d["ndegen"], "hmnr": d["hmnr_ev"]}, 0.0)
    oa = wtin.orbital_atoms(w.nprojs, w.soc)
    got = hrfile.get_hmnr_cell(hr, g.umatrix, oa, w.pos_direct, g.pos_new)
    irv, nd, h = O.get_hmnr_cell(hr["irvec"], hr["ndegen"], hr["hmnr"], g.umatrix, oa, w.pos_direct,
                                 g.pos_new)
    assert np.array_equal(got["irvec"], irv) and np.array_equal(got["hmnr"], h)
    # the (010) hopping of the bulk moves to R' = (0, 0, -1): along -R3' = R2 in this cell
    i = [tuple(v) for v in d["irvec"]].index((0, 1, 0))
    j = [tuple(v) for v in got["irvec"]].index((0, 0, -1))
    assert np.allclose(got["hmnr"][j], hr["hmnr"][i])


@pytest.mark.parametrize("seed", [1, 2])
def test_remap_multi_atom_matches_oracle(tmp_path, seed):
    p = tmp_path / "wt.in"
    p.write_text(WT_IN)
    w = wtin.read_wt_in(p)
    g = wtin.surface_geometry(w)
    hr = _random_hr(w.num_wann, 2, seed)
    oa = wtin.orbital_atoms(w.nprojs, w.soc)
    got = hrfile.get_hmnr_cell(hr, g.umatrix, oa, w.pos_direct, g.pos_new)
    irv, nd, h = O.get_hmnr_cell(hr["irvec"], hr["ndegen"], hr["hmnr"], g.umatrix, oa, w.pos_direct,
                                 g.pos_new)
    assert np.array_equal(got["irvec"], irv) and np.array_equal(got["ndegen"], nd)
    assert np.array_equal(got["hmnr"], h)
    assert len(irv) > 50 and (np.abs(irv) <= 8).all()


def test_remap_identity_equals_surface_cell():
    hr = _random_hr(3, 2, 5)
    a = hrfile.get_hmnr_cell(hr, np.eye(3), np.zeros(3, int), np.zeros((1, 3)), np.zeros((1, 3)))
    b = hrfile.surface_cell(hr)
    assert np.array_equal(a["irvec"], b["irvec"]) and np.array_equal(a["hmnr"], b["hmnr"])
