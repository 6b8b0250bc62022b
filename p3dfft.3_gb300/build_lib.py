"""Builds the GB300 P3DFFT++ libraries in-tree with nvcc (no cmake, no torch extension).

Outputs (git-ignored, rebuilt on each machine):
  p3dfft.3_gb300/lib/libp3dfft_gb300.so   C-ABI library: host runtime + sm_103a kernels
  p3dfft.3_gb300/lib/libp3dfft_mpi1.so    single-rank MPI shim for sample programs

Usage:  python p3dfft.3_gb300/build_lib.py [--force]
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
MAIN_SO = os.path.join(LIB, "libp3dfft_gb300.so")
MPI_SO = os.path.join(LIB, "libp3dfft_mpi1.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC]
CFLAGS += os.environ.get("P3DFFT_GB300_NVCC_FLAGS", "").split()  # extra tuning defines

SOURCES = ["stage_kernels.cu", "core.cpp", "batch.cpp", "serve.cpp", "noalloc.cu"]
# fast_inst.cu once per (arithmetic, kind, part): 0 float-float / 1 FP64 / 2 FP32 / 3 FP32 with
# split twiddles x C2C / R2C / C2R / DCT-I,DST-I / DCT,DST II-IV; the float-float units in two
# halves of the lengths
FAST_UNITS = [(a, k, p) for a in range(4) for k in range(5) for p in range(2 if a == 0 else 1)]
HEADERS = ["kernels.h", "runtime.h", "df_arith.cuh", "stage_common.cuh", "fast_stage.cuh"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INC, h) for h in ("p3dfft.h", "Cwrap.h", "Fwrap.h", "p3dfft_gb300.h", "mpi.h")]
    jobs = []
    objs = []
    units = [(src, src + ".o", []) for src in SOURCES]
    units += [("fast_inst.cu", f"fast_inst_a{a}_k{k}_p{p}.o",
               [f"-DP3D_FAST_ARITH={a}", f"-DP3D_FAST_KIND={k}", f"-DP3D_FAST_PART={p}"])
              for a, k, p in FAST_UNITS]
    for src, obj, defs in units:
        sp = os.path.join(CSRC, src)
        op = os.path.join(OBJ, obj)
        objs.append(op)
        if force or not _newer(op, [sp] + hdrs + [__file__]):
            jobs.append([NVCC] + ARCH + CFLAGS + defs + ["-c", sp, "-o", op])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for _ in ex.map(_run, jobs):
            pass
    if force or jobs or not _newer(MAIN_SO, objs):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", MAIN_SO + ".tmp"] + objs + ["-lpthread", "-ldl", "-lrt"])
        os.replace(MAIN_SO + ".tmp", MAIN_SO)
    mpi_src = os.path.join(CSRC, "mpi_single.c")
    if force or not _newer(MPI_SO, [mpi_src, os.path.join(INC, "mpi.h")]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-I" + INC, "-o", MPI_SO + ".tmp", mpi_src])
        os.replace(MPI_SO + ".tmp", MPI_SO)
    if verbose:
        print("built", MAIN_SO)
    return MAIN_SO


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
