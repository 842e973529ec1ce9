"""A C host links libwtgpu.so directly (no Python): it creates a model, and on a
machine without a GPU gets WTG_ENODEV and the library's error text back, and the
argument checks of the engine and tile calls answer without a device."""
import shutil
import subprocess

import pytest

from wannier_tools_gb300 import _lib

from .conftest import ROOT, has_gpu

C_SRC = r"""
#include <stdio.h>
#include "wtgpu.h"

int main(void) {
  const int irvec[3] = {0, 0, 0};
  const double hmnr[2] = {0.1, 0.0};
  const int ndegen[1] = {1};
  wtg_model_t m = 0;
  char msg[256];
  int rc = wtg_model_create(1, 1, irvec, hmnr, ndegen, 1, 10, &m);
  wtg_last_error(msg, (int)sizeof msg);
  printf("create %d %s\n", rc, msg);
  printf("tile %d\n", wtg_tile_set(WTG_PREC_MIXED, 112, 52));
  printf("graphs %d\n", wtg_engine_set_graphs(0, 1));
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
@pytest.mark.skipif(has_gpu(), reason="checks the no-device answers of a C host")
def test_c_host_links_and_reports(built_lib, tmp_path):
    src = tmp_path / "host.c"
    src.write_text(C_SRC)
    exe = tmp_path / "host"
    lib = _lib.LIB_PATH
    cuda_lib = "/usr/local/cuda/lib64"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        "-o", str(exe), str(lib), f"-L{cuda_lib}", "-lcudart",
                        f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda_lib}"],
                       capture_output=True, text=True)
    if r.returncode != 0 and "cannot find -lcudart" in r.stderr:
        pytest.skip("no CUDA runtime to link against")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = dict(line.split(" ", 1) for line in out.stdout.strip().splitlines())
    rc, msg = lines["create"].split(" ", 1)
    assert int(rc) == _lib.WTG_ENODEV and msg
    assert int(lines["tile"]) == _lib.WTG_EINVAL
    assert int(lines["graphs"]) == _lib.WTG_EINVAL


C_SOLVE = r"""
#include <stdio.h>
#include <stdlib.h>
#include "wtgpu.h"

/* A C host runs a surface spectrum through the C ABI.  The input file holds
   nw np nR nk nomega eta ntop nbot, then irvec (3, nR), HmnR as (re, im) pairs in
   (nw, nw, nR) column-major order, k (nk, 2) column-major, the omegas and the
   two orbital lists; one line per point is printed: dos_l dos_r dos_bulk iters
   status. */
int main(int argc, char** argv) {
  if (argc < 2) return 1;
  FILE* f = fopen(argv[1], "r");
  int nw, np, nr, nk, nom, ntop, nbot;
  double eta;
  if (!f || fscanf(f, "%d %d %d %d %d %lf %d %d", &nw, &np, &nr, &nk, &nom, &eta, &ntop, &nbot) != 8)
    return 2;
  int* irv = malloc(sizeof(int) * 3 * nr);
  double* h = malloc(sizeof(double) * 2 * nw * nw * nr);
  double* k = malloc(sizeof(double) * 2 * nk);
  double* w = malloc(sizeof(double) * nom);
  int* top = malloc(sizeof(int) * ntop);
  int* bot = malloc(sizeof(int) * nbot);
  for (int i = 0; i < 3 * nr; ++i) if (fscanf(f, "%d", &irv[i]) != 1) return 2;
  for (int i = 0; i < 2 * nw * nw * nr; ++i) if (fscanf(f, "%lf", &h[i]) != 1) return 2;
  for (int i = 0; i < 2 * nk; ++i) if (fscanf(f, "%lf", &k[i]) != 1) return 2;
  for (int i = 0; i < nom; ++i) if (fscanf(f, "%lf", &w[i]) != 1) return 2;
  for (int i = 0; i < ntop; ++i) if (fscanf(f, "%d", &top[i]) != 1) return 2;
  for (int i = 0; i < nbot; ++i) if (fscanf(f, "%d", &bot[i]) != 1) return 2;
  fclose(f);
  wtg_model_t m = 0;
  char msg[256];
  int rc = wtg_model_create(nw, nr, irv, h, NULL, np, 10, &m);
  if (rc != WTG_OK) { wtg_last_error(msg, (int)sizeof msg); fprintf(stderr, "%s\n", msg); return 3; }
  const int n = nk * nom;
  double* dl = malloc(sizeof(double) * n);
  double* dr = malloc(sizeof(double) * n);
  double* db = malloc(sizeof(double) * n);
  int32_t* it = malloc(sizeof(int32_t) * n);
  uint8_t* st = malloc(n);
  rc = wtg_surface_spectrum(m, nk, k, nom, w, eta, 1e-16, 100, ntop, top, nbot, bot, 0, WTG_PREC_FP64,
                            dl, dr, db, it, st);
  if (rc < 0) { wtg_last_error(msg, (int)sizeof msg); fprintf(stderr, "%s\n", msg); return 4; }
  for (int i = 0; i < n; ++i) printf("%.17g %.17g %.17g %d %d\n", dl[i], dr[i], db[i], it[i], st[i]);
  wtg_model_destroy(m);
  return 0;
}
"""


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c_host_runs_a_spectrum(built_lib, tmp_path):
    """A C program (no Python in the process) drives a real GPU solve through
    wtg_model_create / wtg_surface_spectrum; its results match the oracle to 1e-9."""
    import numpy as np

    from oracle import wt_oracle as O
    from wannier_tools_gb300 import synthetic
    m = synthetic.make_model(6, 2, seed=31)
    kp = synthetic.random_kpoints(3, seed=2)
    om = np.array([-0.3, 0.05, 0.4]) * O.EV2HARTREE
    eta = 1e-2 * O.EV2HARTREE
    top, bot = [1, 3, 5], [2, 6]
    nr = m.hmnr.shape[0]
    ht = m.hmnr.transpose(0, 2, 1)                       # [R][j][i]: (nw, nw, nR) column-major
    h = np.stack([ht.real, ht.imag], -1).ravel()
    kcol = np.ascontiguousarray(kp.T).ravel()            # (nk, 2) column-major
    with open(tmp_path / "in.txt", "w") as f:
        f.write(f"{m.nw} {m.np_} {nr} {len(kp)} {len(om)} {eta!r} {len(top)} {len(bot)}\n")
        f.write(" ".join(str(int(x)) for x in m.irvec.ravel()) + "\n")
        f.write(" ".join(repr(float(x)) for x in h) + "\n")
        f.write(" ".join(repr(float(x)) for x in kcol) + "\n")
        f.write(" ".join(repr(float(x)) for x in om) + "\n")
        f.write(" ".join(map(str, top)) + "\n" + " ".join(map(str, bot)) + "\n")
    src = tmp_path / "solve.c"
    src.write_text(C_SOLVE)
    exe = tmp_path / "solve"
    lib = _lib.LIB_PATH
    cuda_lib = "/usr/local/cuda/lib64"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        "-o", str(exe), str(lib), f"-L{cuda_lib}", "-lcudart",
                        f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda_lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), str(tmp_path / "in.txt")], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    got = np.array([[float(x) for x in line.split()] for line in out.stdout.strip().splitlines()])
    ref = O.surface_spectrum(m.hmnr, m.irvec, m.ndegen, m.nw, m.np_, kp, om, eta, top, bot)
    # outputs are (nk, nomega) column-major: point i = ik + iw * nk
    for c, name in enumerate(("dos_l", "dos_r", "dos_bulk")):
        want = ref[name].ravel(order="F")
        assert np.max(np.abs(got[:, c] - want) / np.abs(want)) <= 1e-9, name
    assert np.abs(got[:, 3] - ref["iters"].ravel(order="F")).max() <= 1
    assert (got[:, 4] == 0).all()
