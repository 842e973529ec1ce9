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
