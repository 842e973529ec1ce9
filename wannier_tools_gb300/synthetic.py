"""Seeded synthetic tight-binding models for the surface-spectrum workloads.

The reference's headline workloads name models by shape only (Num_wann, Np,
hopping law); no Hamiltonian files exist for them, so they are generated here
from a seed.  The model is written directly in the surface-cell form that
``get_hmnr_cell`` produces for a (001) surface of a cubic lattice with all
orbitals at the origin (identity transform, src/readHmnR.f90:578-766): R
vectors are ordered with R1 fastest, then R2, then R3 (the order of
src/readHmnR.f90:663-674), ``ndegen`` is all ones with 1/ndegen folded into
the values (src/readHmnR.f90:681,720), and energies are converted to Hartree
as readNormalHmnR does (src/readHmnR.f90:155-159).

Hopping law (lattice constant a = 1 Angstrom):
  H(R)_mn = exp(-|R| / 1.2 A) * (x + i y),  x, y ~ N(0, (0.5 eV)^2 / 2)
  H(-R) = H(R)^dagger,
  H(0) Hermitian with onsite energies U(-1, 1) eV on its diagonal.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

EV2HARTREE = 1.0 / 27.211385          # src/module.f90:713


@dataclass
class SurfaceModel:
    """A model in the surface-cell form consumed by ham_qlayer2qlayer."""
    nw: int
    np_: int
    hmnr: np.ndarray        # (nR, nw, nw) complex128, Hartree: hmnr[r, i, j] = H(i, j; R_r)
    irvec: np.ndarray       # (nR, 3) int32
    ndegen: np.ndarray      # (nR,) int32
    seed: int = 0

    @property
    def ndim(self) -> int:
        return self.nw * self.np_

    @property
    def nrpts(self) -> int:
        return int(self.hmnr.shape[0])


def make_model(nw: int, np_: int, seed: int, rmax: int = 3, decay: float = 1.2,
               sigma_ev: float = 0.5, onsite_ev: float = 1.0) -> SurfaceModel:
    """Seeded Hermitian HmnR with R in [-rmax, rmax]^3 (343 vectors for rmax = 3)."""
    rng = np.random.default_rng(seed)
    rs = [(r1, r2, r3) for r3 in range(-rmax, rmax + 1)
          for r2 in range(-rmax, rmax + 1) for r1 in range(-rmax, rmax + 1)]
    index = {r: i for i, r in enumerate(rs)}
    nR = len(rs)
    h = np.zeros((nR, nw, nw), dtype=np.complex128)
    for r in rs:
        neg = (-r[0], -r[1], -r[2])
        if r == (0, 0, 0):
            a = (rng.normal(0.0, sigma_ev / np.sqrt(2.0), (nw, nw))
                 + 1j * rng.normal(0.0, sigma_ev / np.sqrt(2.0), (nw, nw)))
            h0 = 0.5 * (a + a.conj().T)
            h0[np.diag_indices(nw)] = rng.uniform(-onsite_ev, onsite_ev, nw)
            h[index[r]] = h0
        elif r > neg:                       # draw one of each +-R pair
            amp = np.exp(-np.sqrt(r[0] ** 2 + r[1] ** 2 + r[2] ** 2) / decay)
            a = amp * (rng.normal(0.0, sigma_ev / np.sqrt(2.0), (nw, nw))
                       + 1j * rng.normal(0.0, sigma_ev / np.sqrt(2.0), (nw, nw)))
            h[index[r]] = a
            h[index[neg]] = a.conj().T
    irvec = np.array(rs, dtype=np.int32)
    ndegen = np.ones(nR, dtype=np.int32)
    return SurfaceModel(nw=nw, np_=np_, hmnr=h * EV2HARTREE, irvec=irvec, ndegen=ndegen, seed=seed)


def chain_model(eps0_ev: float, t_ev: float) -> SurfaceModel:
    """Single-orbital nearest-neighbour chain along R3 (closed-form surface GF)."""
    irvec = np.array([[0, 0, -1], [0, 0, 0], [0, 0, 1]], dtype=np.int32)
    h = np.zeros((3, 1, 1), dtype=np.complex128)
    h[0, 0, 0] = t_ev
    h[1, 0, 0] = eps0_ev
    h[2, 0, 0] = t_ev
    return SurfaceModel(nw=1, np_=1, hmnr=h * EV2HARTREE, irvec=irvec,
                        ndegen=np.ones(3, np.int32), seed=-1)


def random_kpoints(n: int, seed: int) -> np.ndarray:
    """k uniform over the surface BZ, fractional coordinates in [-0.5, 0.5)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.5, 0.5, (n, 2))
