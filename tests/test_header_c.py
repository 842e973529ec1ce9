"""include/wtgpu.h is plain C: a C99 translation unit that takes the address of
every declared entry point compiles without warnings (the Fortran iso_c_binding
side and C hosts see exactly these prototypes)."""
import shutil
import subprocess

import pytest

from .conftest import ROOT
from .test_abi_cpu import declared_symbols


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_compiles_as_c99(tmp_path):
    names = sorted(declared_symbols())
    src = tmp_path / "use_header.c"
    body = "\n".join(f"  (void)&{n};" for n in names)
    src.write_text('#include "wtgpu.h"\n\nint main(void) {\n' + body + "\n  return 0;\n}\n")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        f"-I{ROOT / 'include'}", "-c", str(src), "-o", str(tmp_path / "u.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
