"""Build recipe for oracle/_ref/libp3dfft_ref.so: the reference library itself, compiled here.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's own build/{init,templ,exec,deriv,wrap}.C,
unchanged and in place under the reference tree (nothing is copied), against:
  - oracle/refshim/p3dfft3config.h   the header configure would generate (FFTW back end, ESTIMATE);
  - oracle/refshim/mpi.h + include/mpi.h, mpi_p2p.c, p3dfft.3_gb300/csrc/mpi_single.c
                                       MPI on a single rank;
  - oracle/refshim/fftw3.h + fftw_shim.c + oracle/p3d_oracle.c
                                       FFTW 3's rank-1 "many" entry points on the oracle's 1D math.
The reference's planner, memory-order reorders, derivative and C/Fortran wrappers therefore run
exactly as written; only FFTW's 1D arithmetic is substituted.  The library exports the
reference's C interface (include/Cwrap.h) and is driven by oracle/pyref.py.

The reference tree is located by $P3DFFT_REFERENCE_DIR; when it is absent (as on a machine
without the reference sources) build() returns None and callers skip.  Output goes only to
oracle/_ref/ (git-ignored).

    python oracle/build_ref.py          # build (incremental)
    python oracle/build_ref.py --force  # rebuild
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SHIM = os.path.join(HERE, "refshim")
OUT = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT, "libp3dfft_ref.so")
REF_SOURCES = ["init", "templ", "exec", "deriv", "wrap"]


def reference_dir():
    d = os.environ.get("P3DFFT_REFERENCE_DIR", "/root/reference")
    return d if os.path.isfile(os.path.join(d, "build", "templ.C")) else None


def _c_sources():
    return [os.path.join(SHIM, "fftw_shim.c"), os.path.join(SHIM, "mpi_p2p.c"), os.path.join(HERE, "p3d_oracle.c"),
            os.path.join(ROOT, "p3dfft.3_gb300", "csrc", "mpi_single.c")]


def _inputs(ref):
    files = [os.path.join(ref, "build", n + ".C") for n in REF_SOURCES]
    files += [os.path.join(ref, "include", h) for h in ("p3dfft.h", "Cwrap.h", "Fwrap.h")]
    files += _c_sources() + [os.path.join(SHIM, f) for f in os.listdir(SHIM)]
    files += [os.path.join(HERE, "p3d_oracle.h"), os.path.join(ROOT, "include", "mpi.h"), os.path.abspath(__file__)]
    return files


def build(force: bool = False):
    """Returns the library path, or None when the reference sources are not present."""
    ref = reference_dir()
    if ref is None:
        return None
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(f) for f in _inputs(ref))):
        return LIB_PATH
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    # Include order: the reference's own headers, then the shims (no p3dfft.h of this repository).
    cxx = ["g++", "-O2", "-fPIC", "-fopenmp", "-std=c++11", "-w", "-DHAVE_CONFIG_H", "-I" + SHIM,
           "-I" + os.path.join(ref, "include")]
    cc = ["gcc", "-O2", "-fPIC", "-fopenmp", "-std=gnu99", "-w", "-I" + SHIM, "-I" + os.path.join(ROOT, "include")]
    jobs = []
    for n in REF_SOURCES:
        jobs.append(cxx + ["-c", os.path.join(ref, "build", n + ".C"), "-o", os.path.join(objdir, n + ".o")])
    for src in _c_sources():
        jobs.append(cc + ["-c", src, "-o", os.path.join(objdir, os.path.basename(src)[:-2] + ".o")])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed: " + " ".join(cmd) + "\n" + r.stderr[-4000:])

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(objdir, n + ".o") for n in REF_SOURCES]
    objs += [os.path.join(objdir, os.path.basename(s)[:-2] + ".o") for s in _c_sources()]
    # -Bsymbolic-functions: the library's internal calls bind to its own definitions even when a process
    # has also loaded libp3dfft_gb300.so (which exports the same C and C++ names).
    run(["g++", "-shared", "-fopenmp", "-Wl,-Bsymbolic-functions", "-o", LIB_PATH + ".tmp"] + objs + ["-lm"])
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    p = build(force="--force" in sys.argv)
    print(p if p else "reference sources not present: nothing built")
