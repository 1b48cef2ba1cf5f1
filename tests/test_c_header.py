"""The C ABI from C (no GPU): ``include/mbem_gb300.h`` compiles as strict
C99, and a C program linked against the library calls entry points whose
answer needs no device (the version, record sizes, argument checks)."""

import os
import shutil
import subprocess

import pytest

from mbem_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "mbem_gb300.h"

int main(void) {
    if (mbem_version() < 1) return 1;
    if (mbem_geom_record_bytes(3) != 3 * 32 * sizeof(float)) return 2;
    /* refused before any launch: no triangles */
    if (mbem_mesh_distance((const float*)0, (const double*)0, 0, (const double*)0, 4, 1.0,
                           (double*)0, (int64_t*)0, (void*)0) != MBEM_ERR_ARG) return 3;
    printf("ok %d\n", mbem_version());
    return 0;
}
"""


@pytest.fixture(scope="module")
def gcc():
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    return cc


def test_header_is_strict_c99(gcc, tmp_path):
    src = tmp_path / "inc.c"
    src.write_text('#include "mbem_gb300.h"\nint main(void) { return 0; }\n')
    subprocess.run([gcc, "-std=c99", "-pedantic", "-Wall", "-Werror", "-fsyntax-only",
                    "-I", os.path.join(ROOT, "include"), str(src)], check=True, capture_output=True)


def test_c_program_links_and_calls_the_library(gcc, tmp_path):
    if not os.path.exists(_native.LIB_PATH):
        from mbem_gb300 import build
        build.build()
    src = tmp_path / "prog.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "prog"
    libdir = os.path.dirname(_native.LIB_PATH)
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lmbem_gb300", f"-Wl,-rpath,{libdir}"], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
