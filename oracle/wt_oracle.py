"""CPU oracle for WannierTools' surface Green's-function path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; it is
used by ``tests/``, by ``__graft_entry__.smoke()`` as the checker, and by the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` as the timed CPU
restatement of the reference.

It restates, in numpy + scipy's LAPACK/BLAS, the exact call sequence of the
reference (quanshengwu/wannier_tools 2.7.1, Fortran 90):

* ``ham_qlayer2qlayer``   src/ham_qlayer2qlayer.f90:45-87  (Fourier sum in iR
  order, then Np x Np block assembly of H00 / H01)
* ``surfgreen_1985``      src/surfgreen.f90:74-134 (Lopez-Sancho 1985
  decimation; same operation order, ``zgesv``-with-identity inverse as in
  src/inverse.f90:43-55, ``zgemm`` as in src/mat_mul.f90:23, ``sum(abs(alpha))``
  convergence test and itermax)
* the spectral sums of ``surfstat``  src/surfstat.f90:149-160 and of
  ``SurfaceDOSkk``  src/fermiarc.f90:237-248, their grids
  (src/surfstat.f90:84-88, src/fermiarc.f90:140-150, 193-194) and output
  transforms (src/surfstat.f90:237-247, src/fermiarc.f90:372-397).
* the spin-resolved sums  src/surfstat.f90:162-192 (six full products with the
  Pauli matrices of src/surfstat.f90:103-114, exactly as the reference does).

Parity status: UNPINNED against outputs of the reference itself.  The
reference ships no golden outputs for this path (its CI only checks that
``wt.x`` runs) and cannot be built in this environment (no Fortran compiler).
The oracle is instead pinned against closed-form known answers (the
semi-infinite 1-D chain, rotated decoupled chains, Np-invariance), see
``tests/test_oracle_kat.py``.  The LAPACK/BLAS used here is scipy's bundled
OpenBLAS; the reference links whatever system LAPACK/BLAS or MKL it was built
with (src/Makefile:42), which no reference test pins either.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.linalg import blas, lapack

# --- constants, restated with the reference's literal values -----------------
PI_REF = 3.14159265358979                    # src/module.f90:719 (truncated literal)
EV2HARTREE = 1.0 / 27.211385                 # src/module.f90:713
ANGSTROM2ATOMIC = 1.0 / 0.529177210903       # src/module.f90:711
EPS9 = float(np.float32(1e-9))               # src/module.f90:728 (single-precision literal)
ACCURACY_REF = float(np.float32(1e-16))      # src/surfgreen.f90:42 (single-precision literal)
ITERMAX_REF = 100                            # src/surfgreen.f90:39
IJMAX_REF = 10                               # src/module.f90:505

# per-point status bits (the reference prints or ignores these conditions)
ST_OK = 0
ST_NOT_CONVERGED = 1        # itermax reached without sum|alpha| <= tol (src/surfgreen.f90:86-123)
ST_SINGULAR = 2             # zgesv info /= 0 (src/inverse.f90:53 prints and continues)
ST_NONFINITE = 4


def ham_qlayer2qlayer(k, hmnr, irvec, ndegen, nw, np_, ijmax=IJMAX_REF):
    """H00/H01 for one in-plane k (fractional surface-BZ coordinates).

    Follows src/ham_qlayer2qlayer.f90:45-87.  ``hmnr`` has shape (nR, nw, nw)
    with ``hmnr[iR, i, j] = HmnR_surfacecell(i+1, j+1, iR+1)`` (Hartree),
    ``irvec`` shape (nR, 3) integer, ``ndegen`` shape (nR,).
    Returns (H00, H01) as (N, N) complex128 arrays, N = nw*np_.
    """
    nR = hmnr.shape[0]
    hij = np.zeros((2 * ijmax + 1, nw, nw), dtype=np.complex128)
    for ir in range(nR):                                  # :48 loop order kept
        ia = float(irvec[ir, 0])
        ib = float(irvec[ir, 1])
        ic = int(irvec[ir, 2])
        if abs(ic) <= ijmax:                              # :54
            kdotr = k[0] * ia + k[1] * ib                 # :55
            ratio = complex(math.cos(2.0 * PI_REF * kdotr), math.sin(2.0 * PI_REF * kdotr))
            hij[ic + ijmax] += hmnr[ir] * ratio / float(ndegen[ir])   # :58-60
    n = nw * np_
    h00 = np.zeros((n, n), dtype=np.complex128)
    h01 = np.zeros((n, n), dtype=np.complex128)
    for i in range(1, np_ + 1):                           # :70-77
        for j in range(1, np_ + 1):
            if abs(i - j) <= ijmax:
                h00[nw * (i - 1):nw * i, nw * (j - 1):nw * j] = hij[(j - i) + ijmax]
    for i in range(1, np_ + 1):                           # :80-87
        for j in range(np_ + 1, 2 * np_ + 1):
            if j - i <= ijmax:
                h01[nw * (i - 1):nw * i, nw * (j - 1 - np_):nw * (j - np_)] = hij[(j - i) + ijmax]
    return h00, h01


VASP_TO_THZ = 29.54263748                    # src/module.f90:1042


def ham_qlayer2qlayer_loto(k, hmnr, irvec, ndegen, nw, np_, born, diele, masses, cell_volume,
                           ijmax=IJMAX_REF):
    """ham_qlayer2qlayer_LOTO (src/ham_qlayer2qlayer.f90:312-476) for an identity
    lattice transform: k moved to (1e-4, 1e-4) when |k|^2 <= 1e-4 (:366-370);
    temp1(qq) = k1 D(qq,1) + k2 D(qq,2), temp2 = k.temp1 (:372-375);
    constant_t = 4*3.1415926/(temp2*V)*VASPToTHZ/0.529177 (:376, the literal
    3.1415926 kept); kBorn(ii,pp) = k1 Z(ii,1,pp) + k2 Z(ii,2,pp) (:378-382);
    nac(i,j) = kBorn(jj,qq) kBorn(ii,pp) constant_t / sqrt(M(ii) M(jj)) added to
    HmnR(:,:,iR) before the phase sum (:395-406).  born (natoms, 3, 3),
    diele (3, 3), masses (natoms,)."""
    kn = [float(k[0]), float(k[1])]
    if abs(kn[0] ** 2 + kn[1] ** 2) <= 0.0001:
        kn = [0.0001, 0.0001]
    z = np.asarray(born, dtype=np.float64)
    d = np.asarray(diele, dtype=np.float64)
    mass = np.asarray(masses, dtype=np.float64)
    natoms = z.shape[0]
    temp1 = [kn[0] * d[q, 0] + kn[1] * d[q, 1] for q in range(2)]
    temp2 = kn[0] * temp1[0] + kn[1] * temp1[1]
    constant_t = 4.0 * 3.1415926 / (temp2 * cell_volume) * VASP_TO_THZ / 0.529177
    kborn = np.array([[kn[0] * z[ii, 0, pp] + kn[1] * z[ii, 1, pp] for pp in range(3)]
                      for ii in range(natoms)])
    nac = np.zeros((nw, nw))
    for ii in range(natoms):
        for pp in range(3):
            for jj in range(natoms):
                for qq in range(3):
                    nac[ii * 3 + pp, jj * 3 + qq] = (kborn[jj, qq] * kborn[ii, pp] * constant_t
                                                     / math.sqrt(mass[ii] * mass[jj]))
    return ham_qlayer2qlayer(kn, np.asarray(hmnr) + nac[None, :, :], irvec, ndegen, nw, np_, ijmax)


def inv(a):
    """src/inverse.f90:1-58: zgesv with an identity right-hand side.

    Returns (A^-1, info).  The reference prints on info /= 0 and continues
    with whatever zgesv left in B; the same array is returned here."""
    n = a.shape[0]
    b = np.asfortranarray(np.eye(n, dtype=np.complex128))
    _lu, _piv, x, info = lapack.zgesv(np.asfortranarray(a), b, overwrite_a=1, overwrite_b=1)
    return x, int(info)


def mat_mul(a, b):
    """src/mat_mul.f90:3-27: C = A*B via ZGEMM('N','N')."""
    return blas.zgemm(1.0, a, b)


# The same two operations in another valid FP64 rounding order, used only to
# measure how far two correct FP64 evaluations of the reference's algorithm
# can lie apart at a point (its FP64 noise floor): the inverse by zgetrf +
# zgetri instead of zgesv with an identity right-hand side, and each product
# with its K sum split in two halves that are added.  Neither is "more
# correct"; a system LAPACK/BLAS other than scipy's (the reference links
# whatever it was built with, src/Makefile:42) differs from the oracle in the
# same way.
def inv_reordered(a):
    lu, piv, info = lapack.zgetrf(np.asfortranarray(a))
    if info != 0:
        return np.eye(a.shape[0], dtype=np.complex128), int(info)
    x, info2 = lapack.zgetri(lu, piv)
    return x, int(info2)


def mat_mul_reordered(a, b):
    h = a.shape[1] // 2
    return blas.zgemm(1.0, a[:, :h], b[:h]) + blas.zgemm(1.0, a[:, h:], b[h:])


def surfgreen_1985(omega, h00, h01, eta, accuracy=ACCURACY_REF, itermax=ITERMAX_REF,
                   reordered=False):
    """Lopez-Sancho (1985) decimation, src/surfgreen.f90:7-137.

    Returns (GLL, GRR, GB, iters, status): iters = iterations executed
    (1..itermax), status a bitmask of ST_* flags.  reordered=True evaluates
    the same steps with inv_reordered / mat_mul_reordered (noise-floor probe)."""
    inv_ = inv_reordered if reordered else inv
    mat_mul_ = mat_mul_reordered if reordered else mat_mul
    n = h00.shape[0]
    ones = np.asfortranarray(np.eye(n, dtype=np.complex128))
    epsiloni = np.asfortranarray(h00.copy())              # :74-78
    epsilons = np.asfortranarray(h00.copy())
    epsilons_t = np.asfortranarray(h00.copy())
    alphai = np.asfortranarray(h01.copy())
    betai = np.asfortranarray(np.conj(h01.T))
    omegac = complex(omega, eta)                          # :82
    status = ST_OK
    iters = 0
    converged = False
    for it in range(1, itermax + 1):                      # :86
        iters = it
        g0, info = inv_(omegac * ones - epsiloni)          # :88-89
        if info != 0:
            status |= ST_SINGULAR
        mat1 = mat_mul_(alphai, g0)                        # :92
        mat2 = mat_mul_(betai, g0)                         # :95
        g0 = mat_mul_(mat1, betai)                         # :98
        epsiloni = epsiloni + g0                           # :99
        epsilons = epsilons + g0                           # :102
        g0 = mat_mul_(mat2, alphai)                        # :107
        epsiloni = epsiloni + g0                           # :108
        epsilons_t = epsilons_t + g0                       # :110
        g0 = mat_mul_(mat1, alphai)                        # :113
        alphai = g0
        g0 = mat_mul_(mat2, betai)                         # :116
        betai = g0
        real_temp = float(np.sum(np.abs(alphai)))          # :120
        if real_temp <= accuracy:                          # :121
            converged = True
            break
    if not converged:
        status |= ST_NOT_CONVERGED
    gll, info = inv_(omegac * ones - epsilons)             # :127-128
    if info != 0:
        status |= ST_SINGULAR
    grr, info = inv_(omegac * ones - epsilons_t)           # :130-131
    if info != 0:
        status |= ST_SINGULAR
    gb, info = inv_(omegac * ones - epsiloni)              # :133-134
    if info != 0:
        status |= ST_SINGULAR
    return gll, grr, gb, iters, status


def spectral_sums(gll, grr, gb, top, bot, nw, scale=1.0):
    """Spectral sums of one (k, omega) point.

    src/surfstat.f90:150-160 (scale 1) and src/fermiarc.f90:238-248
    (each term divided by pi: scale = 1/pi applied per term as the reference
    does).  ``top``/``bot`` are 1-based orbital indices into 1..nw."""
    n = gll.shape[0]
    dl = 0.0
    dr = 0.0
    db = 0.0
    if scale == 1.0:
        for io in top:
            dl = dl - gll[io - 1, io - 1].imag
        for io in bot:
            i = n - nw + io
            dr = dr - grr[i - 1, i - 1].imag
        for i in range(n):
            db = db - gb[i, i].imag
    else:
        for io in top:
            dl = dl - gll[io - 1, io - 1].imag / PI_REF
        for io in bot:
            i = n - nw + io
            dr = dr - grr[i - 1, i - 1].imag / PI_REF
        for i in range(n):
            db = db - gb[i, i].imag / PI_REF
    return dl, dr, db


def spin_matrices(nw, np_):
    """sigma_x/y/z in the |up..up down..down> basis, src/surfstat.f90:103-114."""
    n = nw * np_
    sx = np.zeros((n, n), np.complex128)
    sy = np.zeros((n, n), np.complex128)
    sz = np.zeros((n, n), np.complex128)
    nh = nw // 2
    for i in range(1, np_ + 1):
        for j in range(1, nh + 1):
            a = nw * (i - 1) + j - 1
            b = nw * (i - 1) + j + nh - 1
            sx[a, b] = 1.0
            sx[b, a] = 1.0
            sy[a, b] = -1j
            sy[b, a] = 1j
            sz[a, a] = 1.0
            sz[b, b] = -1.0
    return sx, sy, sz


def spin_sums(gll, grr, top, nw, np_, bot=None, divide_by_pi=False):
    """Spin-resolved sums with six full products G*sigma, as the reference does.

    surfstat (bot=None, src/surfstat.f90:162-192): the right surface also runs
    over TopOrbitals (src/surfstat.f90:178-192), no 1/pi.
    SurfaceDOSkk spin texture (bot given, divide_by_pi, src/fermiarc.f90:272-327):
    the right surface runs over Ndim - Num_wann + BottomOrbitals, each term / pi.
    Returns (sx_l, sy_l, sz_l, sx_r, sy_r, sz_r)."""
    sx, sy, sz = spin_matrices(nw, np_)
    n = gll.shape[0]
    out = []
    for side, g in enumerate((gll, grr)):
        if side == 1 and bot is not None:
            idx = [n - nw + io for io in bot]
        else:
            idx = list(top)
        for s in (sx, sy, sz):
            c = mat_mul(g, s)
            acc = 0.0
            for io in idx:
                if divide_by_pi:
                    acc = acc - c[io - 1, io - 1].imag / PI_REF
                else:
                    acc = acc - c[io - 1, io - 1].imag
            out.append(acc)
    return tuple(out)


# --- drivers ----------------------------------------------------------------

def surfstat_grid(omegamin, omegamax, omeganum):
    """src/surfstat.f90:84-88: eta = 3*(wmax-wmin)/nw, omega excludes wmax."""
    eta = (omegamax - omegamin) / float(omeganum) * 3.0
    omega = np.array([omegamin + (i - 1) * (omegamax - omegamin) / float(omeganum)
                      for i in range(1, omeganum + 1)])
    return omega, eta


def kplane_grid(nk1, nk2, k2d_start, vec1, vec2):
    """src/fermiarc.f90:68-70,140-150: odd-bumped nkx,nky and the k12 list
    (ikp runs j fastest).  Returns (nkx, nky, k12 (nkx*nky, 2), ik12)."""
    nkx = nk1 + 1 if nk1 % 2 == 0 else nk1
    nky = nk2 + 1 if nk2 % 2 == 0 else nk2
    k12 = np.zeros((nkx * nky, 2))
    ik12 = np.zeros((nkx * nky, 2), dtype=np.int64)
    ikp = 0
    for i in range(1, nkx + 1):
        for j in range(1, nky + 1):
            ik12[ikp] = (i, j)
            for c in range(2):
                k12[ikp, c] = (k2d_start[c] + (i - 1) * vec1[c] / float(nkx - 1)
                               + (j - 1) * vec2[c] / float(nky - 1))
            ikp += 1
    return nkx, nky, k12, ik12


def surface_spectrum(hmnr, irvec, ndegen, nw, np_, kpts, omegas, eta, top, bot,
                     scale=1.0, accuracy=ACCURACY_REF, itermax=ITERMAX_REF,
                     ijmax=IJMAX_REF, with_spin=False, loto=None, reordered=False):
    """Loop body of surfstat (src/surfstat.f90:123-197) / SurfaceDOSkk
    (src/fermiarc.f90:206-248) over an explicit (k, omega) list.

    Returns a dict of (nk, nomega) arrays: dos_l, dos_r, dos_bulk, iters,
    status (and sx_l..sz_r when with_spin).  reordered=True: the decimation in
    the other FP64 rounding order (surfgreen_1985's noise-floor probe)."""
    nk = len(kpts)
    nwo = len(omegas)
    out = {name: np.zeros((nk, nwo)) for name in ("dos_l", "dos_r", "dos_bulk")}
    out["iters"] = np.zeros((nk, nwo), np.int32)
    out["status"] = np.zeros((nk, nwo), np.uint8)
    if with_spin:
        for name in ("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r"):
            out[name] = np.zeros((nk, nwo))
    for ik in range(nk):
        if loto is None:
            h00, h01 = ham_qlayer2qlayer(kpts[ik], hmnr, irvec, ndegen, nw, np_, ijmax)
        else:
            h00, h01 = ham_qlayer2qlayer_loto(kpts[ik], hmnr, irvec, ndegen, nw, np_, *loto, ijmax=ijmax)
        for j in range(nwo):
            gll, grr, gb, it, st = surfgreen_1985(omegas[j], h00, h01, eta, accuracy, itermax,
                                                  reordered=reordered)
            dl, dr, db = spectral_sums(gll, grr, gb, top, bot, nw, scale)
            out["dos_l"][ik, j] = dl
            out["dos_r"][ik, j] = dr
            out["dos_bulk"][ik, j] = db
            if not (math.isfinite(dl) and math.isfinite(dr) and math.isfinite(db)):
                st |= ST_NONFINITE
            out["iters"][ik, j] = it
            out["status"][ik, j] = st
            if with_spin:
                s = spin_sums(gll, grr, top, nw, np_, bot=(bot if scale != 1.0 else None),
                              divide_by_pi=(scale != 1.0))
                for name, v in zip(("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r"), s):
                    out[name][ik, j] = v
    return out


def surfstat_post(dos_l, dos_r, dos_bulk):
    """src/surfstat.f90:237-247: log|dos| and the *_only arrays."""
    l_only = dos_l - dos_bulk
    l_only = np.where(l_only < 0, EPS9, l_only)
    r_only = dos_r - dos_bulk
    r_only = np.where(r_only < 0, EPS9, r_only)
    return (np.log(np.abs(dos_l)), np.log(np.abs(dos_r)),
            np.log(np.abs(dos_bulk) + EPS9), l_only, r_only)


def arc_post(dos_l, dos_r):
    """src/fermiarc.f90:372-397: *_only = dos where dos >= max/10, else eps9."""
    l_only = np.where(dos_l < dos_l.max() / 10.0, EPS9, dos_l)
    r_only = np.where(dos_r < dos_r.max() / 10.0, EPS9, dos_r)
    return l_only, r_only


def jdos_kpath(dos):
    """src/surfstat.f90:889-905: along the k path, per omega j and shift
    iq1 = iq - Nk_half (Nk_half = (knv2-1)/2), the sum over
    ik1 in [max(-Nk_half-iq1, -Nk_half)+Nk_half+1, min(Nk_half-iq1, Nk_half)+Nk_half+1]
    of dos(ik1, j)*dos(ik1+iq1, j), accumulated in that order (1-based indices)."""
    d = np.asarray(dos, dtype=np.float64)
    nk, nom = d.shape
    nh = (nk - 1) // 2
    out = np.zeros((nk, nom))
    for j in range(nom):
        col = d[:, j]
        for iq in range(1, nk + 1):
            iq1 = iq - nh
            imin = max(-nh - iq1, -nh) + nh + 1
            imax = min(nh - iq1, nh) + nh + 1
            acc = 0.0
            for ik1 in range(imin, imax + 1):
                acc = acc + float(col[ik1 - 1]) * float(col[ik1 - 1 + iq1])
            out[iq - 1, j] = acc
    return out


def qpi_kplane(chans, p1, p2, scale):
    """src/fermiarc.f90:497-545: for q = (iq1, iq2) in ikp order (i outer,
    j inner, :140-150), sum over ik2 (outer) and ik1 (inner) of
    sum_c in_c(ik1, ik2)*in_c(mod(ik1+iq1-2, p1)+1, mod(ik2+iq2-2, p2)+1),
    the channel products added left to right; times scale (1/(nkx*nky) for
    jdos, :555-556; 1 for jsdos).  Sequential sums: small grids only."""
    arrs = [np.asarray(c, dtype=np.float64) for c in chans]
    nkx, nky = arrs[0].shape
    out = np.zeros(nkx * nky)
    q = 0
    for b1 in range(nkx):
        for b2 in range(nky):
            acc = 0.0
            for a2 in range(nky):
                c2 = (a2 + b2) % p2
                for a1 in range(nkx):
                    c1 = (a1 + b1) % p1
                    term = float(arrs[0][a1, a2]) * float(arrs[0][c1, c2])
                    for a in arrs[1:]:
                        term = term + float(a[a1, a2]) * float(a[c1, c2])
                    acc = acc + term
            out[q] = acc if scale == 1.0 else acc * scale
            q += 1
    return out


def get_hmnr_cell_identity(irvec, ndegen, hmnr, max_ir=8):
    """get_hmnr_cell (src/readHmnR.f90:578-766) for an identity Umatrix with
    every orbital's atom at the same place in both cells, so that
    irvec_new = irvec (:624-634).  Marks rpts_array (:641), orders R' by
    nested loops nir3, nir2, nir1 (:663-674), assigns HmnR/ndegen (:720) and
    sets ndegen_surfacecell = 1 (:681)."""
    rpts = {}
    for ir in range(irvec.shape[0]):
        v = tuple(int(x) for x in irvec[ir])
        if max(abs(v[0]), abs(v[1]), abs(v[2])) > max_ir:
            continue
        rpts[v] = 1
    order = []
    for n3 in range(-max_ir, max_ir + 1):
        for n2 in range(-max_ir, max_ir + 1):
            for n1 in range(-max_ir, max_ir + 1):
                if (n1, n2, n3) in rpts:
                    order.append((n1, n2, n3))
    rmap = {v: i for i, v in enumerate(order)}
    nw = hmnr.shape[1]
    out = np.zeros((len(order), nw, nw), np.complex128)
    for ir in range(irvec.shape[0]):
        v = tuple(int(x) for x in irvec[ir])
        if v not in rmap:
            continue
        for j in range(nw):
            for i in range(nw):
                out[rmap[v], i, j] = hmnr[ir, i, j] / ndegen[ir]
    return np.array(order, np.int32).reshape(-1, 3), np.ones(len(order), np.int32), out


def get_hmnr_cell(irvec, ndegen, hmnr, umatrix, orb_atom, pos_old, pos_new, max_ir=8):
    """get_hmnr_cell (src/readHmnR.f90:578-766) for any SURFACE card, step by step:
    for every (ir, j, i) (:624-645), Rmn = irvec + tau(atom j) - tau(atom i) in the
    original cell (:636), latticetransform (src/ham_qlayer2qlayer.f90:817-838:
    x_c = sum_r Rmn_r Uinv(r, c)), minus tau'(atom j) - tau'(atom i) in the surface
    cell (:638), ANINT (:641-643), the |R'| <= max_ir cut (:645); R' ordered by
    nested loops nir3, nir2, nir1 (:663-674); HmnR/ndegen assigned (a later
    (ir, i, j) replaces an earlier one, :720); ndegen_surfacecell = 1 (:681).
    orb_atom: 0-based atom of each orbital; positions in direct coordinates."""
    uinv = np.linalg.inv(np.asarray(umatrix, dtype=float))
    nw = hmnr.shape[1]

    def anint(x):
        return int(math.copysign(math.floor(abs(x) + 0.5), x))

    def new_r(ir, i, j):
        rmn = [float(irvec[ir][c]) + pos_old[orb_atom[j]][c] - pos_old[orb_atom[i]][c] for c in range(3)]
        x = [sum(rmn[r] * uinv[r][c] for r in range(3)) for c in range(3)]
        return tuple(anint(x[c] - (pos_new[orb_atom[j]][c] - pos_new[orb_atom[i]][c])) for c in range(3))

    rpts = set()
    for ir in range(irvec.shape[0]):
        for j in range(nw):
            for i in range(nw):
                v = new_r(ir, i, j)
                if max(abs(v[0]), abs(v[1]), abs(v[2])) <= max_ir:
                    rpts.add(v)
    order = [(n1, n2, n3) for n3 in range(-max_ir, max_ir + 1) for n2 in range(-max_ir, max_ir + 1)
             for n1 in range(-max_ir, max_ir + 1) if (n1, n2, n3) in rpts]
    rmap = {v: k for k, v in enumerate(order)}
    out = np.zeros((len(order), nw, nw), np.complex128)
    for ir in range(irvec.shape[0]):
        for j in range(nw):
            for i in range(nw):
                v = new_r(ir, i, j)
                if v in rmap:
                    out[rmap[v], i, j] = hmnr[ir, i, j] / ndegen[ir]
    return np.array(order, np.int32).reshape(-1, 3), np.ones(len(order), np.int32), out


def chain_surface_gf(z, e0, t):
    """Closed-form retarded surface and bulk Green's functions of the
    semi-infinite 1-D chain (onsite e0, hopping t): g solves
    t^2 g^2 - (z - e0) g + 1 = 0 with |t g| < 1; G_bulk = 1/(z - e0 - 2 t^2 g)."""
    r = np.sqrt((z - e0) ** 2 - 4.0 * t * t + 0j)
    c = [(z - e0 - r) / (2.0 * t * t), (z - e0 + r) / (2.0 * t * t)]
    g = c[0] if abs(t * c[0]) < abs(t * c[1]) else c[1]
    return g, 1.0 / (z - e0 - 2.0 * t * t * g)
