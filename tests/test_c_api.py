"""The C ABI from a C program (tests/c_api/warp_from_c.c): it compiles and links
against include/idwarp_gb300.h and the built library on the CPU, and runs a
translation warp and reverse product on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_c(tmp_path, built_lib):
    exe = str(tmp_path / "warp_from_c")
    libdir = os.path.dirname(built_lib)
    cmd = ["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_api", "warp_from_c.c"), "-o", exe, "-L", libdir, "-lidwarp_gb300",
           "-Wl,-rpath," + libdir, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_compiles_and_links(tmp_path, built_lib):
    assert os.path.exists(_build_c(tmp_path, built_lib))


@pytest.mark.gpu
def test_c_program_runs(tmp_path, built_lib):
    exe = _build_c(tmp_path, built_lib)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
