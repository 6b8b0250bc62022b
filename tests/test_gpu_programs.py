"""GPU: the drop-in programs in tests/programs (C++ API and C API flows of the reference's sample
programs) compiled against include/ and run on the GPU; each prints the samples' result line
and exits 0 only when every check passes."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "p3dfft.3_gb300", "lib")


def _build_and_run(tmp_path, prog, args):
    cxx = prog.endswith(".cpp")
    cc = "g++" if cxx else "gcc"
    assert shutil.which(cc), cc
    exe = str(tmp_path / "prog")
    cmd = [cc, "-O2", "-I" + INC, os.path.join(ROOT, "tests", "programs", prog), "-L" + LIBDIR, "-lp3dfft_gb300",
           "-lp3dfft_mpi1", "-lm", "-Wl,-rpath," + LIBDIR, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    return r


@pytest.mark.parametrize("dims", [(32, 32, 32), (64, 48, 40)])
def test_cpp_api_program(gpu, tmp_path, dims):
    r = _build_and_run(tmp_path, "cpp_r2c_deriv.cpp", dims)
    assert r.returncode == 0 and "Results are correct" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("dims", [(16, 12, 10), (64, 64, 64)])
def test_c_api_program(gpu, tmp_path, dims):
    r = _build_and_run(tmp_path, "c_api_c2c.c", dims)
    assert r.returncode == 0 and "Results are correct" in r.stdout, r.stdout + r.stderr


def test_fortran_entry_points(gpu, tmp_path):
    """Every *_f entry point (reference build/wrap.C:575-792) called as a compiled Fortran program
    calls it (by reference, 1-based derivative direction, program-owned type-ID variables), each
    bit-identical to the matching C entry point (tests/programs/fortran_abi.c)."""
    r = _build_and_run(tmp_path, "fortran_abi.c", [])
    assert r.returncode == 0 and "Results are correct" in r.stdout, r.stdout + r.stderr
