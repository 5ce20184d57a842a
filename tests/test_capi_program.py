"""Compiled callers of the C ABI without Python: a C++ program performing the
fraunhoferFocal sequence (upload an Armadillo-layout cube, transform, download)
and a C file that includes the header. Compiled here with the system
compilers against csim_gb300/libcsimgpu.so; the program runs on the GPU."""
import os
import shutil
import subprocess

import pytest

from csim_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "capi")
OUT = os.path.join(ROOT, "_build", "capi")


def _compile(cc, src, exe, extra):
    os.makedirs(OUT, exist_ok=True)
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [cc, *extra, "-I" + os.path.join(ROOT, "include"), os.path.join(SRC, src), "-o", exe,
           "-L" + libdir, "-lcsimgpu", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


@pytest.fixture(scope="module")
def program():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    return _compile(cxx, "fraunhofer_focal.cpp", os.path.join(OUT, "fraunhofer_focal"),
                    ["-std=c++17", "-O2"])


def test_header_compiles_as_c_and_links():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = _compile(cc, "header_c.c", os.path.join(OUT, "header_c"), ["-std=c99", "-Wall",
                                                                      "-Werror"])
    assert subprocess.run([exe]).returncode == 0  # csg_version needs no GPU


def test_cpp_program_builds(program):
    assert os.path.exists(program)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,bound", [(6, 1e-6), (16, 2e-7)])
def test_cpp_fraunhofer_focal_sequence(program, precision, bound):
    r = subprocess.run([program, str(bound), str(precision)], capture_output=True, text=True,
                       timeout=120)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
