"""CPU: the C-ABI boundary.

- libp3dfft_gb300.so exports every function declared in include/Cwrap.h, Fwrap.h and
  p3dfft_gb300.h, and the 44 P3DFFT_* type-ID globals with the reference's values;
  libp3dfft_mpi1.so exports every routine of the single-rank include/mpi.h.
- Without a GPU the library fails loudly (error code + message), it has no CPU path.
- The repository's drop-in programs (tests/programs) and, when the reference tree is present,
  the reference's own sample programs compile and link unchanged against include/.
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "p3dfft.3_gb300", "lib")
import refpin  # noqa: E402

REF_SAMPLES = refpin.sample_dir()  # $P3DFFT_REFERENCE_SAMPLES, or the reference tree's sample/

FUNC_RE = re.compile(r"^\s*(?:extern\s+)?[A-Za-z_][\w\s\*]*?\b((?:p3dfft|MPI|find_grid)\w*)\s*\(", re.M)


def declared(header):
    text = open(os.path.join(INC, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return sorted(set(FUNC_RE.findall(text)))


def exported(so):
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if len(line.split()) >= 3}


def test_every_declared_function_is_exported(p3d):
    syms = exported(os.path.join(LIBDIR, "libp3dfft_gb300.so"))
    for h in ("Cwrap.h", "Fwrap.h", "p3dfft_gb300.h"):
        names = declared(h)
        assert names, h
        missing = [n for n in names if n not in syms]
        assert not missing, (h, missing)


def test_mpi_shim_exports(p3d):
    syms = exported(os.path.join(LIBDIR, "libp3dfft_mpi1.so"))
    names = declared("mpi.h")
    assert len(names) >= 20
    assert not [n for n in names if n not in syms]


def test_type_id_globals(p3d):
    lib = p3d.lib()
    lib.p3dfft_setup()
    names = list(p3d.TYPE_IDS.items())
    assert len(names) == 44
    for name, val in names:
        assert ctypes.c_int.in_dll(lib, "P3DFFT_" + name).value == val, name


def test_fails_loudly_without_gpu(p3d):
    lib = p3d.lib()
    p = lib.p3dfft_gb300_device_alloc(16)
    if p:
        lib.p3dfft_gb300_device_free(ctypes.c_void_p(p))
        pytest.skip("a GPU is present")
    lib.p3dfft_clear_error()
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], (8, 8, 8), (0, 1, 2), (5, 8, 8),
                        (1, 2, 0), -1, 0)
    import numpy as np
    with pytest.raises(p3d.P3DFFTError, match="NO_DEVICE"):
        f.exec(np.zeros((8, 8, 8)))


def _compile(src, out, cxx):
    cc = "g++" if cxx else "gcc"
    if shutil.which(cc) is None:
        pytest.skip(cc + " not available")
    cmd = [cc, "-w", "-I" + INC, "-DGIT_VERSION=\"gb300\"", "-DGIT_DATE=\"n/a\""]
    if cxx:
        cmd += ["-std=c++11"]
    cmd += ["-I" + os.path.dirname(src), src, "-L" + LIBDIR, "-lp3dfft_gb300", "-lp3dfft_mpi1", "-lm",
            "-Wl,-rpath," + LIBDIR, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_fortran_module_variables_are_set_by_setup(p3d, tmp_path):
    """A Fortran program's module variables (the type IDs bound by the reference's
    build/fp3dfft++mod.f90) live in the program; p3dfft_setup must fill them in.  The C stand-in
    for that program defines them itself and checks their values (no GPU needed)."""
    exe = str(tmp_path / "fabi")
    _compile(os.path.join(ROOT, "tests", "programs", "fortran_abi.c"), exe, False)
    r = subprocess.run([exe, "ids"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Results are correct" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("prog", ["cpp_r2c_deriv.cpp", "c_api_c2c.c", "fortran_abi.c"])
def test_own_programs_compile(p3d, tmp_path, prog):
    _compile(os.path.join(ROOT, "tests", "programs", prog), str(tmp_path / "a.out"), prog.endswith(".cpp"))


CPP_SAMPLES = ["test3D_r2c", "test_deriv", "test1D_cos", "test1D_sin", "test3D_c2c", "test3D_c2c_inplace",
               "test3D_r2c_single", "test1D_cos_complex", "test_transplan", "bench_c2c"]
C_SAMPLES = ["test3D_r2c", "test_deriv", "test1D_cos", "test1D_r2c", "test2D+empty", "test3D_c2c",
             "test3D_c2c_inplace", "test3D_r2c_memord", "test3D_r2c_single", "test1D_cos_complex"]


@pytest.mark.skipif(REF_SAMPLES is None, reason="reference sample programs not present")
@pytest.mark.parametrize("name,cxx", [(n, True) for n in CPP_SAMPLES] + [(n, False) for n in C_SAMPLES])
def test_reference_samples_compile_unchanged(p3d, tmp_path, name, cxx):
    src = os.path.join(REF_SAMPLES, "C++" if cxx else "C", name + (".C" if cxx else ".c"))
    _compile(src, str(tmp_path / "s.out"), cxx)
