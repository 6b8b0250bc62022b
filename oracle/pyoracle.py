"""ctypes binding of the CPU oracle (oracle/p3d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg as the checker.  The product library never imports this module.

The oracle restates the reference pipeline (build/templ.C planner, build/exec.C executor,
build/deriv.C derivative, FFTW's published transform definitions) in plain C; see the header of
p3d_oracle.c for the line-by-line citations.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libp3d_oracle.so")

# FFTW r2r kinds, in the order of the C enum
REDFT00, REDFT10, REDFT01, REDFT11, RODFT00, RODFT10, RODFT01, RODFT11 = range(8)
K_EMPTY, K_R2C, K_C2R, K_C2C_FWD, K_C2C_BWD, K_R2R = range(6)


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP when available) into oracle/_build/."""
    src = os.path.join(HERE, "p3d_oracle.c")
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src),
                                                  os.path.getmtime(os.path.join(HERE, "p3d_oracle.h")))):
        return LIB_PATH
    base = ["gcc", "-O3", "-fPIC", "-shared", "-std=gnu99", "-o", LIB_PATH + ".tmp", src, "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True, capture_output=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class Grid(ctypes.Structure):
    _fields_ = [("gdims", ctypes.c_int * 3), ("mo", ctypes.c_int * 3), ("dcs", ctypes.c_int)]

    @staticmethod
    def make(gdims, mo, dcs=-1):
        g = Grid()
        for i in range(3):
            g.gdims[i] = int(gdims[i])
            g.mo[i] = int(mo[i])
        g.dcs = int(dcs)
        return g


class Stage(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("dim", ctypes.c_int), ("g1", Grid), ("g2", Grid)]


class Plan3D(ctypes.Structure):
    _fields_ = [("nstages", ctypes.c_int), ("st", Stage * 4), ("L", ctypes.c_int * 3),
                ("dt1", ctypes.c_int), ("dt2", ctypes.c_int), ("prec", ctypes.c_int), ("ok", ctypes.c_int)]


class TypeInfo(ctypes.Structure):
    _fields_ = [("dt1", ctypes.c_int), ("dt2", ctypes.c_int), ("prec", ctypes.c_int),
                ("kind", ctypes.c_int), ("r2r", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.orc_dft_c2c.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        _lib.orc_dft_direct.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        _lib.orc_dft_r2c.argtypes = [ctypes.c_int, dp, dp]
        _lib.orc_dft_c2r.argtypes = [ctypes.c_int, dp, dp]
        _lib.orc_r2r.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        _lib.orc_plan3d_make.argtypes = [ctypes.POINTER(ctypes.c_int * 3), ctypes.POINTER(Grid),
                                         ctypes.POINTER(Grid), ctypes.POINTER(Plan3D)]
        _lib.orc_exec3d.argtypes = [ctypes.POINTER(Plan3D), dp, dp, ctypes.c_int, ctypes.c_int]
        _lib.orc_exec_stage.argtypes = [ctypes.POINTER(Stage), dp, dp, ctypes.c_int, ctypes.c_int]
        _lib.orc_exec_stage_lines.argtypes = [ctypes.POINTER(Stage), dp, dp, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_longlong, ctypes.c_longlong]
        _lib.orc_compute_deriv.argtypes = [ctypes.POINTER(Grid), dp, dp, ctypes.c_int]
        _lib.orc_compute_deriv_axis.argtypes = [ctypes.POINTER(Grid), dp, dp, ctypes.c_int, ctypes.c_int]
        _lib.orc_type_info_get.argtypes = [ctypes.c_int, ctypes.POINTER(TypeInfo)]
        _lib.orc_set_batched.argtypes = [ctypes.c_int]
        _lib.orc_swap0.argtypes = [ctypes.POINTER(ctypes.c_int * 3), ctypes.POINTER(ctypes.c_int * 3), ctypes.c_int]
        _lib.orc_find_order.argtypes = [ctypes.POINTER(ctypes.c_int * 3), ctypes.POINTER(Grid),
                                        ctypes.POINTER(Grid), ctypes.POINTER(ctypes.c_int * 3)]
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _as_f64(a) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(a.astype(np.complex128)).view(np.float64)
    return np.ascontiguousarray(a, dtype=np.float64)


# ---- 1D ----------------------------------------------------------------------------------
def dft_c2c(x, sign=-1, direct=False):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n = x.size
    out = np.empty(n, np.complex128)
    f = lib().orc_dft_direct if direct else lib().orc_dft_c2c
    f(n, sign, _dp(x.view(np.float64)), _dp(out.view(np.float64)))
    return out


def dft_r2c(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(x.size // 2 + 1, np.complex128)
    lib().orc_dft_r2c(x.size, _dp(x), _dp(out.view(np.float64)))
    return out


def dft_c2r(x, n):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    assert x.size == n // 2 + 1
    out = np.empty(n, np.float64)
    lib().orc_dft_c2r(n, _dp(x.view(np.float64)), _dp(out))
    return out


def r2r(kind, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_r2r(kind, x.size, _dp(x), _dp(out))
    return out


def type_info(tid):
    t = TypeInfo()
    if lib().orc_type_info_get(tid, ctypes.byref(t)) != 0:
        raise ValueError(tid)
    return dict(dt1=t.dt1, dt2=t.dt2, prec=t.prec, kind=t.kind, r2r=t.r2r)


def swap0(mo, L):
    a = (ctypes.c_int * 3)(*mo)
    b = (ctypes.c_int * 3)()
    lib().orc_swap0(ctypes.byref(b), ctypes.byref(a), L)
    return tuple(b)


# ---- 3D ----------------------------------------------------------------------------------
def storage_shape(gdims, mo):
    """numpy shape (slowest first) of a field stored with memory order mo."""
    sd = [0, 0, 0]
    for i in range(3):
        sd[mo[i]] = gdims[i]
    return (sd[2], sd[1], sd[0])


def set_batched(on: bool):
    """Stages of C2C lines and of even-length R2C / C2R lines on the batched line engine (True,
    the default) or line by line (False); the same results to rounding."""
    lib().orc_set_batched(1 if on else 0)


class OraclePlan:
    def __init__(self, types, gdims1, mo1, gdims2, mo2, dcs1=-1, dcs2=-1):
        self.types = tuple(int(t) for t in types)
        self.g1 = Grid.make(gdims1, mo1, dcs1)
        self.g2 = Grid.make(gdims2, mo2, dcs2)
        self.p = Plan3D()
        t = (ctypes.c_int * 3)(*self.types)
        self.rc = lib().orc_plan3d_make(ctypes.byref(t), ctypes.byref(self.g1), ctypes.byref(self.g2),
                                        ctypes.byref(self.p))
        if self.rc < 0:
            raise ValueError("oracle planner rejected the transform")

    def stages(self):
        out = []
        for i in range(self.p.nstages):
            s = self.p.st[i]
            out.append(dict(type=s.type, dim=s.dim,
                            gdims1=tuple(s.g1.gdims), mo1=tuple(s.g1.mo), dcs1=s.g1.dcs,
                            gdims2=tuple(s.g2.gdims), mo2=tuple(s.g2.mo), dcs2=s.g2.dcs))
        return out

    @property
    def order(self):
        return tuple(self.p.L)

    def exec(self, x, idir=-1, nthreads=0):
        """x: numpy array (real or complex) holding the input field in storage order."""
        xin = _as_f64(x)
        n_out = self.g2.gdims[0] * self.g2.gdims[1] * self.g2.gdims[2]
        if self.p.dt2 == 2:
            out = np.empty(n_out, np.complex128)
            ov = out.view(np.float64)
        else:
            out = np.empty(n_out, np.float64)
            ov = out
        rc = lib().orc_exec3d(ctypes.byref(self.p), _dp(xin), _dp(ov), int(idir), int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle exec failed rc={rc}")
        return out.reshape(storage_shape(tuple(self.g2.gdims), tuple(self.g2.mo)))


def exec_stage(type_id, dim, gdims1, mo1, gdims2, mo2, x, deriv=False, nthreads=0):
    st = Stage()
    st.type = type_id
    st.dim = dim
    st.g1 = Grid.make(gdims1, mo1)
    st.g2 = Grid.make(gdims2, mo2)
    ti = type_info(type_id)
    xin = _as_f64(x)
    n_out = int(np.prod(gdims2))
    out = np.empty(n_out, np.complex128 if ti["dt2"] == 2 else np.float64)
    ov = out.view(np.float64) if ti["dt2"] == 2 else out
    rc = lib().orc_exec_stage(ctypes.byref(st), _dp(xin), _dp(ov), int(deriv), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle stage failed rc={rc}")
    return out.reshape(storage_shape(gdims2, mo2))


def compute_deriv(x, gdims, mo, dcs, idir, ref_axis=False):
    """ref_axis=True: the storage axis the reference differentiates along (build/deriv.C:89-93)."""
    g = Grid.make(gdims, mo, dcs)
    xin = _as_f64(x)
    out = np.empty(int(np.prod(gdims)), np.complex128)
    rc = lib().orc_compute_deriv_axis(ctypes.byref(g), _dp(xin), _dp(out.view(np.float64)), int(idir),
                                      int(bool(ref_axis)))
    if rc != 0:
        raise RuntimeError("oracle compute_deriv failed")
    return out.reshape(storage_shape(gdims, mo))


_SHARED = {}


def _shared_buf(key, n):
    b = _SHARED.get(key)
    if b is None or b.size < n:
        b = np.random.default_rng(7).uniform(-1, 1, n) if key == "in" else np.empty(n, np.float64)
        _SHARED[key] = b
    return b


def stage_lines_runner(stage: dict, nthreads=0):
    """Returns (run(line0, line1, deriv), bytes_in, bytes_out, nlines) for timing a bounded sample
    of one stage of a plan (stage dicts as returned by OraclePlan.stages()).  All runners share
    one input and one output buffer sized for the largest stage."""
    st = Stage()
    st.type = stage["type"]
    st.dim = stage["dim"]
    st.g1 = Grid.make(stage["gdims1"], stage["mo1"], stage["dcs1"])
    st.g2 = Grid.make(stage["gdims2"], stage["mo2"], stage["dcs2"])
    ti = type_info(stage["type"])
    n1 = int(np.prod(stage["gdims1"])) * ti["dt1"]
    n2 = int(np.prod(stage["gdims2"])) * ti["dt2"]
    inb = _shared_buf("in", n1)
    outb = _shared_buf("out", n2)
    L = stage["dim"]
    nlines = int(np.prod([stage["gdims1"][i] for i in range(3) if i != L]))

    def run(line0, line1, deriv=False):
        rc = lib().orc_exec_stage_lines(ctypes.byref(st), _dp(inb), _dp(outb), int(deriv), int(nthreads),
                                        int(line0), int(line1))
        if rc != 0:
            raise RuntimeError("oracle stage failed")

    return run, n1 * 8, n2 * 8, nlines
