"""Generate the committed fixtures under tests/golden/.

Run from the repository root with the path of a reference checkout (it
reads examples/3DWeyl-model/Weyl3D_hr.dat from it):

    python tests/golden/make_golden.py <path of the wannier_tools checkout>

Fixtures:
  weyl3d_hr_model.npz    the reference's 2-band Weyl model (examples/3DWeyl-model/
                         Weyl3D_hr.dat, eV), parsed as readNormalHmnR does.
  weyl3d_wt.in           the same example's surface-state input file
                         (examples/3DWeyl-model/wt.in-surfacestates), copied
                         unchanged: the drop-in test runs it.
  analytic_chain.npz     closed-form surface / bulk Green's functions of the
                         semi-infinite chain (independent of any code here).
  oracle_weyl3d.npz      oracle outputs (H00/H01 at one k; dos_l/dos_r/dos_bulk
                         and iteration counts on a k x omega grid) for the Weyl
                         model in the (001) surface cell with Np = 2, using
                         surfstat's grid and eta (src/surfstat.f90:84-88).
  oracle_synth_n8.npz    oracle outputs for a seeded synthetic model
                         (Num_wann = 4, Np = 2, Ndim = 8).
The oracle fixtures pin regressions of the oracle and give the GPU tests
reference values that do not need scipy; they are not outputs of the
reference program, which cannot be built here.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import wt_oracle as O  # noqa: E402
from wannier_tools_gb300 import hrfile, synthetic  # noqa: E402

HERE = Path(__file__).resolve().parent


def copy_inputs(ref_root: str) -> None:
    src = Path(ref_root) / "examples/3DWeyl-model/wt.in-surfacestates"
    (HERE / "weyl3d_wt.in").write_text(src.read_text())


def main(ref_root: str) -> None:
    copy_inputs(ref_root)
    hr = hrfile.read_hr(Path(ref_root) / "examples/3DWeyl-model/Weyl3D_hr.dat")
    np.savez(HERE / "weyl3d_hr_model.npz", irvec=hr["irvec"], ndegen=hr["ndegen"], hmnr_ev=hr["hmnr"])

    # closed-form chain
    e0_ev, t_ev = 0.3, 1.0
    e0, t = e0_ev * O.EV2HARTREE, t_ev * O.EV2HARTREE
    omegas = np.linspace(-3.0, 3.0, 13) * O.EV2HARTREE
    etas = np.array([1e-2, 1e-3]) * O.EV2HARTREE
    gs = np.zeros((len(etas), len(omegas)), np.complex128)
    gbk = np.zeros_like(gs)
    for a, eta in enumerate(etas):
        for b, w in enumerate(omegas):
            gs[a, b], gbk[a, b] = O.chain_surface_gf(complex(w, eta), e0, t)
    np.savez(HERE / "analytic_chain.npz", e0_ev=e0_ev, t_ev=t_ev, omegas=omegas, etas=etas,
             g_surface=gs, g_bulk=gbk)

    # Weyl model in the surface cell, Np = 2
    hh = hrfile.to_hartree(hr, 0.0)
    irv, nd, h = O.get_hmnr_cell_identity(hh["irvec"], hh["ndegen"], hh["hmnr"])
    nw, np_ = hr["nw"], 2
    kpath = np.array([[-0.5, 0.0], [-0.2, 0.1], [0.0, 0.0], [0.31, -0.25]])
    omega, eta = O.surfstat_grid(-1.6 * O.EV2HARTREE, 1.6 * O.EV2HARTREE, 16)
    top = [1, 2]
    bot = [1, 2]
    res = O.surface_spectrum(h, irv, nd, nw, np_, kpath, omega, eta, top, bot)
    h00, h01 = O.ham_qlayer2qlayer(kpath[1], h, irv, nd, nw, np_)
    np.savez(HERE / "oracle_weyl3d.npz", irvec_sc=irv, ndegen_sc=nd, hmnr_sc=h, np_=np_, kpath=kpath,
             omega=omega, eta=eta, top=top, bot=bot, h00=h00, h01=h01, **res)

    # seeded synthetic model, Ndim = 8
    m = synthetic.make_model(4, 2, seed=7)
    kp = synthetic.random_kpoints(3, seed=11)
    om = np.linspace(-0.8, 0.8, 5) * O.EV2HARTREE
    eta2 = 1e-2 * O.EV2HARTREE
    res2 = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, kp, om, eta2, [1, 3], [2, 4])
    g = O.surfgreen_1985(om[2], *O.ham_qlayer2qlayer(kp[0], m.hmnr, m.irvec, m.ndegen, m.nw, m.np_), eta2)
    np.savez(HERE / "oracle_synth_n8.npz", nw=4, np_=2, seed=7, kpts=kp, omega=om, eta=eta2,
             top=[1, 3], bot=[2, 4], gll=g[0], grr=g[1], gb=g[2], g_iters=g[3], **res2)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the wannier_tools checkout>")
    main(sys.argv[1])
