"""ctypes driver of the reference library built here (oracle/_ref/libp3dfft_ref.so).

TEST INFRASTRUCTURE ONLY.  The library is the reference's own build/{init,templ,exec,deriv,wrap}.C,
compiled unchanged by oracle/build_ref.py, with only FFTW's 1D arithmetic substituted (the oracle's,
through oracle/refshim/fftw_shim.c).  This module calls it through the reference's C interface
(include/Cwrap.h; build/wrap.C:90-571): p3dfft_setup, p3dfft_init_proc_grid (1x1x1),
p3dfft_init_data_grid, p3dfft_init_3Dtype, p3dfft_plan_3Dtrans, p3dfft_exec_3Dtrans_*,
p3dfft_exec_3Dderiv_*, p3dfft_plan_1Dtrans, p3dfft_exec_1Dtrans_* and p3dfft_compute_deriv_*.

Used by tests/ to pin the oracle and the GPU path to the reference itself, and by
tests/golden/make_ref_golden.py to write the reference's outputs as fixtures.  It is unavailable
(available() is False) where the reference sources are absent.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build_ref  # noqa: E402

MPI_COMM_WORLD = 0x44000000  # include/mpi.h

_lib = None
_pgrid = None


def available() -> bool:
    return build_ref.reference_dir() is not None


def lib():
    global _lib, _pgrid
    if _lib is not None:
        return _lib
    path = build_ref.build()
    if path is None:
        raise RuntimeError("reference sources not present: oracle/_ref cannot be built")
    L = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    ip = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    sig = {
        "p3dfft_setup": ([], None),
        "p3dfft_cleanup": ([], None),
        "p3dfft_init_proc_grid": ([ip, ctypes.c_int], ctypes.c_int),
        "p3dfft_init_data_grid": ([ip, ctypes.c_int, ctypes.c_int, ip, ip], vp),
        "p3dfft_free_data_grid": ([vp], None),
        "p3dfft_init_3Dtype": ([ip], ctypes.c_int),
        "p3dfft_plan_3Dtrans": ([vp, vp, ctypes.c_int], ctypes.c_int),
        "p3dfft_exec_3Dtrans_double": ([ctypes.c_int, vp, vp, ctypes.c_int], None),
        "p3dfft_exec_3Dtrans_single": ([ctypes.c_int, vp, vp, ctypes.c_int], None),
        "p3dfft_exec_3Dderiv_double": ([ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int], None),
        "p3dfft_exec_3Dderiv_single": ([ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int], None),
        "p3dfft_plan_1Dtrans": ([vp, vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_exec_1Dtrans_double": ([ctypes.c_int, vp, vp, ctypes.c_int], None),
        "p3dfft_exec_1Dtrans_single": ([ctypes.c_int, vp, vp, ctypes.c_int], None),
        "p3dfft_compute_deriv_double": ([vp, vp, vp, ctypes.c_int], None),
        "p3dfft_compute_deriv_single": ([vp, vp, vp, ctypes.c_int], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    L.p3dfft_setup()
    _pgrid = L.p3dfft_init_proc_grid((ctypes.c_int * 3)(1, 1, 1), MPI_COMM_WORLD)
    _lib = L
    return L


def reset():
    """p3dfft_cleanup() then p3dfft_setup() and a fresh 1x1x1 processor grid.

    The reference keeps one process-wide FFTW plan cache whose key omits the r2r kind
    (build/templ.C:1243-1261), so an r2r plan made earlier in the process can stand in for a later
    one of another kind with the same length and batch; cleanup() empties it (build/init.C:827-900).
    Plans and grids made before a reset must not be used after it."""
    global _pgrid
    L = lib()
    L.p3dfft_cleanup()
    L.p3dfft_setup()
    _pgrid = L.p3dfft_init_proc_grid((ctypes.c_int * 3)(1, 1, 1), MPI_COMM_WORLD)


def _i3(v):
    return (ctypes.c_int * 3)(*[int(x) for x in v])


def storage_shape(gdims, mo):
    sd = [0, 0, 0]
    for i in range(3):
        sd[mo[i]] = gdims[i]
    return (sd[2], sd[1], sd[0])


def type_prec_dt(tid):
    """(precision bytes, dt1, dt2) of a 1D type ID (build/init.C:121-731)."""
    import pyoracle
    t = pyoracle.type_info(tid)
    return t["prec"], t["dt1"], t["dt2"]


class DataGrid:
    """p3dfft_init_data_grid on the 1x1x1 processor grid; the Grid struct stays owned by the
    reference library until free()."""

    def __init__(self, gdims, mo, dcs=-1):
        L = lib()
        self.gdims = tuple(int(g) for g in gdims)
        self.mo = tuple(int(m) for m in mo)
        self.dcs = int(dcs)
        self.ptr = L.p3dfft_init_data_grid(_i3(gdims), self.dcs, _pgrid, _i3((0, 1, 2)), _i3(mo))
        if not self.ptr:
            raise RuntimeError("reference rejected the data grid")

    def shape(self):
        return storage_shape(self.gdims, self.mo)

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.p3dfft_free_data_grid(self.ptr)
            self.ptr = None


def _buffer(shape, complex_, prec):
    if complex_:
        return np.zeros(shape, np.complex128 if prec == 8 else np.complex64)
    return np.zeros(shape, np.float64 if prec == 8 else np.float32)


def _as(x, complex_, prec):
    if complex_:
        return np.ascontiguousarray(x, dtype=np.complex128 if prec == 8 else np.complex64)
    return np.ascontiguousarray(x, dtype=np.float64 if prec == 8 else np.float32)


class RefPlan3D:
    """transform3D<T1,T2> planned by the reference (p3dfft_plan_3Dtrans)."""

    def __init__(self, types, gdims1, mo1, gdims2, mo2, dcs1=-1, dcs2=-1):
        L = lib()
        self.types = tuple(int(t) for t in types)
        self.g1 = DataGrid(gdims1, mo1, dcs1)
        self.g2 = DataGrid(gdims2, mo2, dcs2)
        t3 = L.p3dfft_init_3Dtype(_i3(self.types))
        self.plan = L.p3dfft_plan_3Dtrans(self.g1.ptr, self.g2.ptr, t3)
        precs = {type_prec_dt(t)[0] for t in self.types}
        if len(precs) != 1:
            raise ValueError("mixed precisions")
        self.prec = precs.pop()
        # element kinds of the ends: the first stage's input and the last stage's output
        dts = [type_prec_dt(t)[1:] for t in self.types]
        self.c_in = any(d[0] == 2 for d in dts) and not any(d == (1, 2) for d in dts)
        self.c_out = any(d[1] == 2 for d in dts) and not any(d == (2, 1) for d in dts)

    def exec(self, x, idir=-1, OW=0):
        L = lib()
        xin = _as(x, self.c_in, self.prec).reshape(self.g1.shape())
        out = _buffer(self.g2.shape(), self.c_out, self.prec)
        f = L.p3dfft_exec_3Dtrans_double if self.prec == 8 else L.p3dfft_exec_3Dtrans_single
        if idir >= 0:
            fd = L.p3dfft_exec_3Dderiv_double if self.prec == 8 else L.p3dfft_exec_3Dderiv_single
            fd(self.plan, xin.ctypes.data, out.ctypes.data, int(idir), int(OW))
        else:
            f(self.plan, xin.ctypes.data, out.ctypes.data, int(OW))
        return out


class RefPlan1D:
    """transplan<T1,T2> planned by the reference (p3dfft_plan_1Dtrans)."""

    def __init__(self, type_id, dim, gdims1, mo1, gdims2, mo2, dcs1=-1, dcs2=-1):
        L = lib()
        self.type_id = int(type_id)
        self.g1 = DataGrid(gdims1, mo1, dcs1)
        self.g2 = DataGrid(gdims2, mo2, dcs2)
        self.plan = L.p3dfft_plan_1Dtrans(self.g1.ptr, self.g2.ptr, self.type_id, int(dim))
        self.prec, dt1, dt2 = type_prec_dt(self.type_id)
        self.c_in, self.c_out = dt1 == 2, dt2 == 2

    def exec(self, x, OW=0):
        L = lib()
        xin = _as(x, self.c_in, self.prec).reshape(self.g1.shape())
        out = _buffer(self.g2.shape(), self.c_out, self.prec)
        f = L.p3dfft_exec_1Dtrans_double if self.prec == 8 else L.p3dfft_exec_1Dtrans_single
        f(self.plan, xin.ctypes.data, out.ctypes.data, int(OW))
        return out


def compute_deriv(x, gdims, mo, dcs, idir, prec=8):
    """compute_deriv<T> through p3dfft_compute_deriv_* (build/deriv.C:85-184, wrap.C:551-568)."""
    L = lib()
    g = DataGrid(gdims, mo, dcs)
    xin = _as(x, True, prec).reshape(g.shape())
    out = _buffer(g.shape(), True, prec)
    f = L.p3dfft_compute_deriv_double if prec == 8 else L.p3dfft_compute_deriv_single
    f(xin.ctypes.data, out.ctypes.data, g.ptr, int(idir))
    return out
