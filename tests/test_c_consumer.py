"""The C ABI from plain C: every public header compiles as pedantic C99 (and C++11),
and a C99 program linked against liboic_gpu.so calls the host-side entry points and
creates a context -- which, on a host without a GPU, must fail with OIC_ERR_CUDA rather
than crash (tests/c_consumer.c).  CPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

INC = os.path.join(ROOT, "include")
HEADERS = ("oic_gpu.h", "oic_ovfile.h", "oic_seqdb.h")


@pytest.mark.parametrize("header", HEADERS)
@pytest.mark.parametrize("lang", [["gcc", "-std=c99", "-pedantic", "-x", "c"], ["g++", "-std=c++11", "-x", "c++"]])
def test_public_header_compiles(header, lang, tmp_path):
    if not shutil.which(lang[0]):
        pytest.skip(lang[0] + " not found")
    src = tmp_path / "h.c"
    src.write_text(f'#include "{header}"\nint main(void) {{ return 0; }}\n')
    r = subprocess.run(lang + ["-Wall", "-Wextra", "-Werror", "-I" + INC, "-fsyntax-only", str(src)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


def test_c_program_uses_the_library(built, tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    lib_dir = os.path.dirname(built["lib"])
    exe = str(tmp_path / "c_consumer")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-I" + INC, os.path.join(ROOT, "tests", "c_consumer.c"), "-o", exe,
                        "-L" + lib_dir, "-loic_gpu", "-Wl,-rpath," + lib_dir], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    r = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() in ("ok create=0", "ok create=3")   # OIC_OK with a GPU, OIC_ERR_CUDA without
    assert sorted(os.listdir(tmp_path / "asm.ovlStore")) == ["0001-001", "index", "info", "statistics"]
