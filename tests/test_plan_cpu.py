"""Host-side launch arithmetic (wannier_tools_gb300/csrc/wtg_plan.h) on the CPU.

The per-model spectrum path splits its k list into chunks whose instance count
kc * nomega, plus one extra work-counter ticket per persistent CTA, must stay a
valid 32-bit int; a chunk's H00/H01 must fit the 8 GiB buffer and the Fourier
kernel's grid.  The header is plain C++, so it is compiled here with g++ and
driven over edge cases (no GPU)."""
import ctypes as C
import shutil
import subprocess

import pytest

from wannier_tools_gb300 import _lib

from .conftest import ROOT

INT_MAX = 2**31 - 1
H_CHUNK = 8 << 30
DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "wtg_plan.h"
int main(int argc, char** argv) {
  for (int i = 1; i + 3 < argc; i += 4) {
    const long long nk = atoll(argv[i]), nom = atoll(argv[i + 1]), n = atoll(argv[i + 2]),
                    g = atoll(argv[i + 3]);
    printf("%d\n", wtg::spectrum_kchunk(nk, nom, n, g, (size_t)8 << 30));
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def kchunk(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("plan")
    (d / "drv.cpp").write_text(DRIVER)
    exe = d / "drv"
    subprocess.run(["g++", "-O1", "-std=c++17", f"-I{ROOT / 'wannier_tools_gb300' / 'csrc'}",
                    str(d / "drv.cpp"), "-o", str(exe)], check=True)

    def run(cases):
        args = [str(v) for c in cases for v in c]
        out = subprocess.run([str(exe), *args], check=True, capture_output=True, text=True).stdout
        return [int(x) for x in out.split()]
    return run


def test_kchunk_bounds(kchunk):
    cases = [
        (40401, 1, 112, 152),          # the Fermi-arc plane: two chunks (8 GiB of H00/H01)
        (101, 201, 40, 608),           # a k-path x omega spectrum
        (10**6, 4097, 8, 152),         # many k x many omega: the 32-bit instance bound binds
        (10**6, 1, 8, 152),            # tiny Ndim: the Fourier grid bound binds
        (10**5, 1, 320, 152),          # large Ndim: the 8 GiB H00/H01 buffer binds
        (5, INT_MAX - 152, 16, 152),   # one k point of the largest omega list that fits
        (5, INT_MAX - 151, 16, 152),   # one omega too many: no chunk
        (0, 1, 16, 152), (1, 0, 16, 152), (1, 1, 0, 152), (1, 1, 16, 0),
    ]
    got = kchunk(cases)
    for (nk, nom, n, g), kc in zip(cases, got):
        if min(nk, nom, n, g) < 1 or nom > INT_MAX - g:
            assert kc == 0, (nk, nom, n, g)
            continue
        assert 1 <= kc <= nk
        assert kc * nom + g <= INT_MAX, (nk, nom, n, g, kc)        # instances + tickets fit int
        assert kc <= 65535 * 8                                        # Fourier grid.z
        assert kc == 1 or kc * 32 * n * n <= H_CHUNK                  # H00/H01 buffer
        # the chunk is the largest that meets every bound
        bound = min(nk, 65535 * 8, max(1, H_CHUNK // (32 * n * n)), (INT_MAX - g) // nom)
        assert kc == bound, (nk, nom, n, g, kc, bound)
    assert got[0] == H_CHUNK // (32 * 112 * 112) == 21399 and got[1] == 101
    assert got[2] == (INT_MAX - 152) // 4097 and got[3] == 65535 * 8
    assert got[4] == H_CHUNK // (32 * 320 * 320)


def test_test_option_arguments(built_lib):
    lib = built_lib
    assert lib.wtg_test_option(0, 1) == _lib.WTG_EINVAL
    assert lib.wtg_test_option(99, 1) == _lib.WTG_EINVAL
    assert lib.wtg_test_option(_lib.TEST_MIXED_SPIN_LIMIT, -1) == _lib.WTG_EINVAL
    assert "negative" in _lib.last_error() or "< 0" in _lib.last_error()
    for opt in (_lib.TEST_FP64_GLOBAL_INVERSE, _lib.TEST_MIXED_SPIN_LIMIT):
        assert lib.wtg_test_option(opt, 3) == _lib.WTG_OK
        assert lib.wtg_test_option(opt, 0) == _lib.WTG_OK
    assert C.sizeof(C.c_int) == 4
