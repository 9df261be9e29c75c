"""include/bsfit.h is a C header: a C99 program that includes it, references
every entry point it declares and calls the ones that need no GPU compiles
with -std=c99 -pedantic -Werror, links against libbsfit.so and runs."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from test_library import _declared_symbols


def test_header_is_c99_and_every_symbol_links(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    from bsfit import build
    lib = build.build()
    names = _declared_symbols()
    refs = ",\n  ".join(f"(fn){n}" for n in names)
    src = f"""#include <stdio.h>
#include "bsfit.h"
typedef void (*fn)(void);
static const fn every_entry[] = {{
  {refs}
}};
int main(void) {{
  printf("%s|%d|%d|%s\\n", bsfit_version(), bsfit_num_params(8),
         (int)(sizeof(every_entry) / sizeof(every_entry[0])), bsfit_status_str(BSFIT_E_INIT_P));
  return bsfit_num_params(3) == 0 ? 0 : 1;
}}
"""
    c = tmp_path / "abi.c"
    c.write_text(src)
    exe = tmp_path / "abi"
    libdir = os.path.dirname(lib)
    r = subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe),
                        "-L", libdir, "-lbsfit", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    version, nv8, count, msg = out.stdout.strip().split("|")
    assert nv8 == "8" and int(count) == len(names) and "initP" in msg
