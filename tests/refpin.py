"""Shared by the tests that pin results to the reference itself and by the golden-vector maker.

- Case tables: the 1D / 3D transforms, memory-order pairs and grids the pin covers.
- A model of the reference's known defects, each checked against the reference built here
  (oracle/_ref) by tests/test_ref_pin.py:
    D1  find_m overwrites a 1D plan's input order with swap0(mo1, dim) when neither order leads
        with the transform dim (build/templ.C:1015-1023); exec then reads the input in that order.
    D2  an EMPTY complex stage with unchanged order that leads with its dim copies half the field
        (memcpy of prec*dims bytes, build/exec.C:555-556).
    D3  reorder_out's (0,2,1) branch re-reads one row per cache block (pin/pout reset from
        pin1/pout1, which never advance; build/exec.C:2006-2016): rows are dropped whenever a
        block holds more than one row.
    D4  exec_deriv calls the derivative exec of every stage whose trans_dim is idir, including an
        EMPTY reorder stage, whose exec is NULL: the process crashes (build/exec.C:173-176, 447).
    D5  reorder_deriv's TRANS_OUT scheme with relative change (1,2,0) gives a wrong derivative
        (build/exec.C:1666-1706).
    D6  the process-wide FFTW plan cache omits the r2r kind (build/templ.C:1243-1261): an r2r
        stage reuses an earlier r2r plan of another kind with the same N, m, strides and dists.
    D7  compute_deriv differentiates along storage axis imo[idir] (build/deriv.C:89-93).
  D1 and D7 are deterministic, and the library reproduces them by default
  (p3dfft_gb300_set_reference_compat); D2-D6 give partly undefined or crashing results and are not
  reproduced.
- fingerprint(): a size-independent digest (seeded sample values, seeded +-1 projections, norm)
  used to compare full-size outputs against the reference's without storing them.
"""
from __future__ import annotations

import itertools

import numpy as np

PERMS = list(itertools.permutations(range(3)))

# 1D type IDs (build/init.C:121-731)
EMPTY_D, EMPTY_DC = 1, 3
R2C_S, R2C_D, C2R_S, C2R_D = 4, 5, 6, 7
C2C_FS, C2C_FD, C2C_BS, C2C_BD = 8, 9, 10, 11
DCT1_RD, DCT1_CD = 13, 15
DST1_RD = 17
DCT2_RD, DCT2_CD = 21, 23
DST2_RD, DST2_CD = 25, 27
DCT3_RD = 29


def storage_shape(gdims, mo):
    sd = [0, 0, 0]
    for i in range(3):
        sd[mo[i]] = gdims[i]
    return (sd[2], sd[1], sd[0])


def inv_mo(mo):
    r = [0, 0, 0]
    for i in range(3):
        r[mo[i]] = i
    return tuple(r)


def rel_change(imo1, imo2):
    """mc of build/exec.C:2268-2296 (imo2[mc[i]] = imo1[i])."""
    a, b = imo1, imo2
    mc = [0, 0, 0]
    mc[2] = (1 if b[1] == a[2] else 0) if b[2] != a[2] else 2
    mc[1] = (0 if b[0] == a[1] else 2) if b[1] != a[1] else 1
    mc[0] = (1 if b[1] == a[0] else 2) if b[0] != a[0] else 0
    return tuple(mc)


def swap0(mo, L):
    """build/templ.C:816-858"""
    t = list(mo)
    if t[L] == 1:
        j = t.index(0)
        t[j] = 1
        t[L] = 0
    elif t[L] == 2:
        t = [(v + 1) % 3 for v in t]
    return tuple(t)


def kind_of(tid):
    """0 EMPTY, 1 R2C, 2 C2R, 3 C2C fwd, 4 C2C bwd, 5 r2r"""
    if tid < 4:
        return 0
    if tid < 12:
        return 1 + (tid - 4) // 2
    return 5


def prec_of(tid):
    if tid < 4:
        return 8 if tid & 1 else 4
    return 8 if (tid - (4 if tid < 12 else 12)) & 1 else 4


def dt_of(tid):
    """(dt1, dt2): 1 real, 2 complex"""
    k = kind_of(tid)
    if k == 0:
        return (2, 2) if tid >= 2 else (1, 1)
    if k == 1:
        return (1, 2)
    if k == 2:
        return (2, 1)
    if k in (3, 4):
        return (2, 2)
    return (2, 2) if (tid - 12) % 4 >= 2 else (1, 1)


def grids_1d(tid, dim, gd):
    g1, g2 = list(gd), list(gd)
    if kind_of(tid) == 1:
        g2[dim] = gd[dim] // 2 + 1
    if kind_of(tid) == 2:
        g1[dim] = gd[dim] // 2 + 1
    return tuple(g1), tuple(g2)


def grids_3d(types, gd):
    """(gdims1, dcs1, gdims2, dcs2) of a 3D plan whose R2C / C2R stage is along dim 0."""
    g1, g2, dcs1, dcs2 = list(gd), list(gd), -1, -1
    if R2C_S in types or R2C_D in types:
        g2[0] = gd[0] // 2 + 1
        dcs2 = 0
    if C2R_S in types or C2R_D in types:
        g1[0] = gd[0] // 2 + 1
        dcs1 = 0
    return tuple(g1), dcs1, tuple(g2), dcs2


# ---- defect model --------------------------------------------------------------------------
def d1_reinterprets(tid, dim, mo1, mo2):
    return kind_of(tid) != 0 and mo1[dim] != 0 and mo2[dim] != 0


def d2_half_copy(tid, dim, mo1, mo2):
    return tid in (2, 3) and tuple(mo1) == tuple(mo2) and mo1[dim] == 0


def d3_reorder_out_021(tid, mo1, mo2):
    return kind_of(tid) == 0 and tuple(mo1) != tuple(mo2) and rel_change(inv_mo(mo1), inv_mo(mo2)) == (0, 2, 1)


def d4_deriv_crash(stages, idir):
    return any(kind_of(s["type"]) == 0 and s["dim"] == idir for s in stages)


def d5_deriv_stage_defect(stages, idir):
    for s in stages:
        if s["dim"] != idir or kind_of(s["type"]) == 0:
            continue
        a, b, L = s["mo1"], s["mo2"], idir
        if a[L] != 0 and b[L] == 0 and rel_change(inv_mo(a), inv_mo(b)) == (1, 2, 0):
            return True
    return False


def ref_1d_sound(tid, dim, mo1, mo2):
    """True when the reference's 1D transplan gives the transform's defined result."""
    return not (d1_reinterprets(tid, dim, mo1, mo2) or d2_half_copy(tid, dim, mo1, mo2)
                or d3_reorder_out_021(tid, mo1, mo2))


def seeded(shape, seed, complex_, prec=8):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, shape)
    if complex_:
        x = x + 1j * rng.uniform(-1, 1, shape)
        return np.ascontiguousarray(x.astype(np.complex128 if prec == 8 else np.complex64))
    return np.ascontiguousarray(x.astype(np.float64 if prec == 8 else np.float32))


# ---- size-independent digest ---------------------------------------------------------------
FP_SAMPLES = 1024
FP_PROJ = 4
_CHUNK = 1 << 23


def fingerprint(a, seed=1234):
    """Seeded sample values, FP_PROJ projections onto +-1 vectors, and the L2 norm of a flat
    array (complex or real), computed in chunks so 1 GB fields need no large temporaries."""
    flat = np.ascontiguousarray(a).reshape(-1)
    n = flat.size
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(n, size=min(FP_SAMPLES, n), replace=False))
    proj = np.zeros(FP_PROJ, np.complex128)
    nrm2 = 0.0
    for c0 in range(0, n, _CHUNK):
        blk = flat[c0:c0 + _CHUNK].astype(np.complex128 if np.iscomplexobj(flat) else np.float64)
        nrm2 += float(np.vdot(blk, blk).real)
        for p in range(FP_PROJ):
            w = np.random.default_rng([seed, p, c0 // _CHUNK]).integers(0, 2, blk.size, dtype=np.int8)
            proj[p] += (blk * (2.0 * w - 1.0)).sum()
    return {"idx": idx, "val": flat[idx].astype(np.complex128), "proj": proj, "norm": np.sqrt(nrm2)}


def fingerprint_error(fa, fb):
    """max(relative L2 of the samples, |projection difference| / norm): both ~ the relative L2
    error of the full arrays for errors spread over the field."""
    assert np.array_equal(fa["idx"], fb["idx"])
    e1 = np.linalg.norm(fa["val"] - fb["val"]) / max(np.linalg.norm(fb["val"]), 1e-300)
    e2 = np.max(np.abs(fa["proj"] - fb["proj"])) / max(fb["norm"], 1e-300)
    return max(e1, e2, abs(fa["norm"] - fb["norm"]) / max(fb["norm"], 1e-300))


# ---- the reference's sample programs, run unchanged ----------------------------------------
# name -> (path under the reference's sample/ directory, input file it reads, its contents).
# Grids are cubes: the samples' forward checks index storage coordinates with the logical dims.
_IN3 = "32 32 32 2 2\n"
SAMPLES = {
    "C++/test3D_r2c": ("C++/test3D_r2c.C", "stdin", _IN3),
    "C++/test3D_c2c": ("C++/test3D_c2c.C", "stdin", "16 16 16 2 2\n"),
    "C++/test3D_c2c_inplace": ("C++/test3D_c2c_inplace.C", "stdin", "16 16 16 2 2\n"),
    "C++/test3D_r2c_single": ("C++/test3D_r2c_single.C", "stdin", _IN3),
    "C++/test_deriv": ("C++/test_deriv.C", "stdin", "32 32 32 2 2 1\n"),
    "C++/bench_c2c": ("C++/bench_c2c.C", "stdin", "16 16 16 2 2\n"),
    "C++/test1D_cos": ("C++/test1D_cos.C", "trans.in", "16 16 16 0 2\n0 1 2\n1 2 0\n"),
    "C++/test1D_sin": ("C++/test1D_sin.C", "trans.in", "16 16 16 1 2\n0 1 2\n2 0 1\n"),
    "C++/test1D_cos_complex": ("C++/test1D_cos_complex.C", "trans.in", "16 16 16 0 2\n0 1 2\n0 1 2\n"),
    "C++/test_transplan": ("C++/test_transplan.C", "trans.in", "16 16 16 0 2\n0 1 2\n1 2 0\n"),
    "C/test3D_r2c": ("C/test3D_r2c.c", "stdin", _IN3),
    "C/test3D_c2c": ("C/test3D_c2c.c", "stdin", "16 16 16 2 2\n"),
    "C/test3D_c2c_inplace": ("C/test3D_c2c_inplace.c", "stdin", "16 16 16 2 2\n"),
    "C/test3D_r2c_single": ("C/test3D_r2c_single.c", "stdin", _IN3),
    "C/test_deriv": ("C/test_deriv.c", "stdin", "32 32 32 2 2 2\n"),
    "C/test2D+empty": ("C/test2D+empty.c", "stdin", _IN3),
    "C/test3D_r2c_memord": ("C/test3D_r2c_memord.c", "memord3d", "32 32 32 2 2\n2 1 0\n1 2 0\n"),
    "C/test1D_cos": ("C/test1D_cos.c", "trans.in", "16 16 16 0 2\n0 1 2\n1 2 0\n"),
    "C/test1D_r2c": ("C/test1D_r2c.c", "trans.in", "16 16 16 0 2\n0 1 2\n1 2 0\n"),
    "C/test1D_cos_complex": ("C/test1D_cos_complex.c", "trans.in", "16 16 16 0 2\n0 1 2\n0 1 2\n"),
}


def sample_dir():
    """The reference's sample/ directory: $P3DFFT_REFERENCE_SAMPLES, else sample/ under the
    reference tree oracle/build_ref.py uses; None when absent."""
    import os
    d = os.environ.get("P3DFFT_REFERENCE_SAMPLES")
    if d and os.path.isdir(d):
        return d
    try:
        import build_ref
    except ImportError:
        return None
    ref = build_ref.reference_dir()
    return os.path.join(ref, "sample") if ref and os.path.isdir(os.path.join(ref, "sample")) else None


def run_sample(name, target, workdir, timeout=300):
    """Compiles sample `name` unchanged and runs it in workdir with its input file written there.
    target "ref": against the reference's headers and oracle/_ref/libp3dfft_ref.so (CPU);
    target "gb300": against include/ and p3dfft.3_gb300/lib (GPU)."""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sd = sample_dir()
    rel_path, fname, text = SAMPLES[name]
    src = os.path.join(sd, rel_path)
    cxx = src.endswith(".C")
    cmd = ["g++" if cxx else "gcc", "-w", "-O1", '-DGIT_VERSION="gb300"', '-DGIT_DATE="n/a"',
           "-I" + os.path.dirname(src)]
    if cxx:
        cmd.append("-std=c++11")
    if target == "ref":
        import build_ref
        lib = os.path.dirname(build_ref.build())
        cmd += ["-DHAVE_CONFIG_H", "-I" + os.path.join(root, "oracle", "refshim"),
                "-I" + os.path.join(build_ref.reference_dir(), "include"), src, "-L" + lib, "-lp3dfft_ref"]
    else:
        lib = os.path.join(root, "p3dfft.3_gb300", "lib")
        cmd += ["-I" + os.path.join(root, "include"), src, "-L" + lib, "-lp3dfft_gb300", "-lp3dfft_mpi1"]
    exe = os.path.join(workdir, "sample.out")
    cmd += ["-lm", "-lstdc++", "-Wl,-rpath," + lib, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return r
    with open(os.path.join(workdir, fname), "w") as f:
        f.write(text)
    with open(os.path.join(workdir, "dims"), "w") as f:
        f.write("1 1\n")
    return subprocess.run([exe], cwd=workdir, capture_output=True, text=True, timeout=timeout)


def sample_passed(r, name):
    """Exit status 0, no "incorrect" result line, and at least one "Results are correct" line
    (bench_c2c's final result line is commented out in its source: it needs its timing line)."""
    out = r.stdout or ""
    if r.returncode != 0 or "incorrect" in out:
        return False
    if name.endswith("bench_c2c"):
        return "Transform time" in out
    return "Results are correct" in out


def det_field(shape, seed, complex_, prec=8):
    """Portable seeded U[-1,1) field (SplitMix64 of the element index; no generator-version
    dependence), used for inputs whose outputs are stored as fixtures."""
    n = int(np.prod(shape)) * (2 if complex_ else 1)
    z = np.arange(n, dtype=np.uint64) + np.uint64((seed * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        z = z * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53) * 2.0 - 1.0
    if complex_:
        x = (u[0::2] + 1j * u[1::2]).reshape(shape)
        return np.ascontiguousarray(x.astype(np.complex128 if prec == 8 else np.complex64))
    return np.ascontiguousarray(u.reshape(shape).astype(np.float64 if prec == 8 else np.float32))


def input_is_complex(types):
    """A 3D plan's input is complex unless one stage is R2C or every stage is real."""
    if any(kind_of(t) == 1 for t in types):
        return False
    return any(dt_of(t)[0] == 2 for t in types)
