"""Python mirror of the P3DFFT++ interface over libp3dfft_gb300.so (ctypes, C ABI only).

Mirrors the reference's C++ objects (include/p3dfft.h): `setup`/`cleanup`, the type-ID
constants, `Transform3D` (transform3D<T1,T2>: plan in the constructor, `exec` / `exec_deriv`),
`TransPlan` (transplan<T1,T2>) and `compute_deriv`.  Arrays are numpy arrays (host memory,
staged through HBM by the library) or objects exposing a CUDA pointer (torch CUDA tensors, or an
int device address), used in place.

There is no CPU path: if the shared library is missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libp3dfft_gb300.so")

# Type IDs: registration order of p3dfft::setup() (reference build/init.C:121-731)
EMPTY_TYPE_SINGLE, EMPTY_TYPE_DOUBLE, EMPTY_TYPE_SINGLE_COMPLEX, EMPTY_TYPE_DOUBLE_COMPLEX = 0, 1, 2, 3
R2CFFT_S, R2CFFT_D, C2RFFT_S, C2RFFT_D = 4, 5, 6, 7
CFFT_FORWARD_S, CFFT_FORWARD_D, CFFT_BACKWARD_S, CFFT_BACKWARD_D = 8, 9, 10, 11
_FAMILIES = ["DCT1", "DST1", "DCT2", "DST2", "DCT3", "DST3", "DCT4", "DST4"]
TYPE_IDS = {
    "EMPTY_TYPE_SINGLE": 0, "EMPTY_TYPE_DOUBLE": 1, "EMPTY_TYPE_SINGLE_COMPLEX": 2,
    "EMPTY_TYPE_DOUBLE_COMPLEX": 3, "R2CFFT_S": 4, "R2CFFT_D": 5, "C2RFFT_S": 6, "C2RFFT_D": 7,
    "CFFT_FORWARD_S": 8, "CFFT_FORWARD_D": 9, "CFFT_BACKWARD_S": 10, "CFFT_BACKWARD_D": 11,
}
for _f, _fam in enumerate(_FAMILIES):
    for _v, _suf in enumerate(["REAL_S", "REAL_D", "COMPLEX_S", "COMPLEX_D"]):
        TYPE_IDS[f"{_fam}_{_suf}"] = 12 + 4 * _f + _v
globals().update(TYPE_IDS)

ERR_NAMES = {0: "OK", 1: "BAD_ARG", 2: "UNSUPPORTED", 3: "CUDA", 4: "NO_DEVICE", 5: "TOO_LARGE", 6: "PLAN",
             7: "ALIGN"}


class P3DFFTError(RuntimeError):
    pass


_lib = None


def lib():
    """Loads the C-ABI library (built by build_lib.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise P3DFFTError(f"{LIB_PATH} is missing: run `python p3dfft.3_gb300/build_lib.py` "
                          "(or __graft_entry__.build()) first")
    L = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    ip = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    sig = {
        "p3dfft_setup": ([], None), "p3dfft_cleanup": ([], None),
        "p3dfft_last_error": ([], ctypes.c_int), "p3dfft_last_error_string": ([], ctypes.c_char_p),
        "p3dfft_clear_error": ([], None),
        "p3dfft_gb300_set_stream": ([vp], None), "p3dfft_gb300_set_sync": ([ctypes.c_int], None),
        "p3dfft_gb300_set_host_direct": ([ctypes.c_int], None),
        "p3dfft_gb300_set_host_pipeline": ([ctypes.c_int], None),
        "p3dfft_gb300_get_host_pipeline": ([], ctypes.c_int),
        "p3dfft_gb300_set_link_ctas": ([ctypes.c_int], None),
        "p3dfft_gb300_get_link_ctas": ([], ctypes.c_int),
        "p3dfft_gb300_set_pageable_direct": ([ctypes.c_int], None),
        "p3dfft_gb300_get_pageable_direct": ([], ctypes.c_int),
        "p3dfft_gb300_set_fp64_arith": ([ctypes.c_int], None), "p3dfft_gb300_get_fp64_arith": ([], ctypes.c_int),
        "p3dfft_gb300_set_reference_compat": ([ctypes.c_int], None),
        "p3dfft_gb300_get_reference_compat": ([], ctypes.c_int),
        "p3dfft_gb300_set_ff_intermediates": ([ctypes.c_int], None),
        "p3dfft_gb300_get_ff_intermediates": ([], ctypes.c_int),
        "p3dfft_gb300_set_fp32_split_twiddles": ([ctypes.c_int], None),
        "p3dfft_gb300_get_fp32_split_twiddles": ([], ctypes.c_int),
        "p3dfft_gb300_set_fp32_tma": ([ctypes.c_int], None),
        "p3dfft_gb300_get_fp32_tma": ([], ctypes.c_int),
        "p3dfft_gb300_device_status": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_inject_tma_stall": ([], None),
        "p3dfft_gb300_tma_launch_count": ([], ctypes.c_longlong),
        "p3dfft_gb300_plan3d": ([ip, ip, ip, ctypes.c_int, ip, ip, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_exec3d": ([ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_destroy3d": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_plan3d_types": ([ctypes.c_int, ip, ip, ip], ctypes.c_int),
        "p3dfft_gb300_plan3d_stages": ([ctypes.c_int, ip, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_plan3d_exec_stages": ([ctypes.c_int, ip, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_plan1d": ([ctypes.c_int, ip, ip, ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_exec1d": ([ctypes.c_int, vp, vp, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_destroy1d": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_compute_deriv": ([ctypes.c_int, vp, vp, ip, ip, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_kernel_count": ([], ctypes.c_longlong), "p3dfft_gb300_reset_kernel_count": ([], None),
        "p3dfft_gb300_enable_timers": ([ctypes.c_int], None), "p3dfft_gb300_timer": ([ctypes.c_int], ctypes.c_double),
        "p3dfft_gb300_reset_timers": ([], None),
        "p3dfft_gb300_device_alloc": ([ctypes.c_longlong], vp), "p3dfft_gb300_device_free": ([vp], None),
        "p3dfft_gb300_memcpy_h2d": ([vp, vp, ctypes.c_longlong], ctypes.c_int),
        "p3dfft_gb300_memcpy_d2h": ([vp, vp, ctypes.c_longlong], ctypes.c_int),
        "p3dfft_gb300_synchronize": ([], ctypes.c_int), "p3dfft_gb300_sm_count": ([], ctypes.c_int), "p3dfft_gb300_version": ([], ctypes.c_char_p),
        "p3dfft_gb300_host_alloc_pinned": ([ctypes.c_longlong], vp), "p3dfft_gb300_host_free_pinned": ([vp], None),
        "p3dfft_gb300_exec3d_noalloc": ([ctypes.c_int, vp, vp, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_noalloc_max_field_bytes": ([], ctypes.c_longlong),
        "p3dfft_gb300_event_record": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_event_elapsed_ms": ([ctypes.c_int, ctypes.c_int], ctypes.c_double),
        "p3dfft_gb300_profile_stages": ([ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_double), ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_create": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_add": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_set_graph": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_set_grouped": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_groups": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_exec": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_batch_kernels": ([ctypes.c_int], ctypes.c_longlong),
        "p3dfft_gb300_batch_field_bytes": ([ctypes.c_int], ctypes.c_double),
        "p3dfft_gb300_batch_destroy": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_server_create": ([ctypes.c_longlong, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_preload_kernels": ([], ctypes.c_int),
        "p3dfft_gb300_set_autotune": ([ctypes.c_int], None),
        "p3dfft_gb300_autotune": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_plan_tuning": ([ctypes.c_int, ctypes.c_int, ip, ip, ctypes.POINTER(ctypes.c_double),
                                      ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_plan_set_engine": ([ctypes.c_int] * 5, ctypes.c_int),
        "p3dfft_gb300_tune_cache_save": ([ctypes.c_char_p], ctypes.c_int),
        "p3dfft_gb300_tune_cache_load": ([ctypes.c_char_p], ctypes.c_int),
        "p3dfft_gb300_tune_cache_clear": ([], None),
        "p3dfft_gb300_server_submit": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp,
                                        ctypes.c_double], ctypes.c_int),
        "p3dfft_gb300_server_wait": ([ctypes.c_int, ctypes.c_int, ctypes.c_double], ctypes.c_int),
        "p3dfft_gb300_server_inject_alloc_failure": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_server_drain": ([ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_server_clock": ([ctypes.c_int], ctypes.c_double),
        "p3dfft_gb300_server_job_times": ([ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "p3dfft_gb300_server_stats": ([ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int], ctypes.c_int),
        "p3dfft_gb300_server_destroy": ([ctypes.c_int], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _i3(v):
    return (ctypes.c_int * 3)(*[int(x) for x in v])


def check(rc=None):
    code = lib().p3dfft_last_error()
    if (rc is not None and rc != 0) or code != 0:
        msg = lib().p3dfft_last_error_string().decode()
        lib().p3dfft_clear_error()
        raise P3DFFTError(f"{ERR_NAMES.get(code, code)}: {msg}")


def setup():
    lib().p3dfft_setup()


def cleanup():
    lib().p3dfft_cleanup()


def set_fp64_arith(mode: int):
    """0: native FP64 (DFMA); 1: float-float on the FP32 pipe."""
    lib().p3dfft_gb300_set_fp64_arith(int(mode))


def set_reference_compat(on: bool):
    """True (default): compute_deriv's axis choice and the 1D input-order reinterpretation of the
    reference (build/deriv.C:89-93, build/templ.C:1015-1023), so results equal the reference's;
    False: the corrected behaviours (differentiate along logical dim idir; read 1D inputs in their
    declared memory order)."""
    lib().p3dfft_gb300_set_reference_compat(1 if on else 0)


def set_ff_intermediates(on: bool):
    """Float-float FP64 stages pass intermediate fields as scaled float-float pairs (True, the
    default) or as IEEE doubles (False)."""
    lib().p3dfft_gb300_set_ff_intermediates(1 if on else 0)


def set_fp32_split_twiddles(on: bool):
    """FP32 stages of FFT length 512-2048 use split (compensated) twiddle products (True, the
    default) or plain FP32 twiddles (False)."""
    lib().p3dfft_gb300_set_fp32_split_twiddles(1 if on else 0)


def set_fp32_tma(on: bool):
    """FP32 C2C / R2C stages with contiguous lines load their tiles by TMA (True, the default)
    or by per-thread global loads (False)."""
    lib().p3dfft_gb300_set_fp32_tma(1 if on else 0)


def get_fp32_tma() -> bool:
    return bool(lib().p3dfft_gb300_get_fp32_tma())


def device_status(clear: bool = True) -> int:
    """Nonzero after a kernel's bounded wait ran out (synchronous); clear resets it."""
    return int(lib().p3dfft_gb300_device_status(1 if clear else 0))


def tma_launch_count() -> int:
    return int(lib().p3dfft_gb300_tma_launch_count())


def inject_tma_stall():
    """Test hook: the next TMA-staged launch's waits run out (20 ms) and set the status word."""
    lib().p3dfft_gb300_inject_tma_stall()


def get_reference_compat() -> bool:
    return bool(lib().p3dfft_gb300_get_reference_compat())


def set_sync(sync: bool):
    lib().p3dfft_gb300_set_sync(1 if sync else 0)


def set_host_direct(on):
    """Page-locked host arrays read / written by the kernels over NVLink-C2C (True, or "in" /
    "out" for one side only) or staged through HBM (False)."""
    mode = {True: 1, False: 0, "in": 2, "out": 3}[on]
    lib().p3dfft_gb300_set_host_direct(mode)


def set_host_pipeline(on: bool):
    """Staged host copies overlapped with the first / last two stages, slab by slab (True, the
    default) or with the first / last stage only (False)."""
    lib().p3dfft_gb300_set_host_pipeline(1 if on else 0)


def get_host_pipeline() -> bool:
    return bool(lib().p3dfft_gb300_get_host_pipeline())


def set_link_ctas(n: int):
    """n > 0: the end stage that reads / writes a page-locked host array directly runs on at
    most n persistent CTAs, slab by slab, with its neighbour stage beside it; 0: stage after
    stage; n < 0: the default (one CTA per SM for FP64, two per SM for FP32)."""
    lib().p3dfft_gb300_set_link_ctas(int(n))


def get_link_ctas() -> int:
    return int(lib().p3dfft_gb300_get_link_ctas())


def set_pageable_direct(on: bool):
    """Pageable host arrays read / written in place by the end stages where the device walks the
    host's page tables (True), or staged through HBM (False, the default)."""
    lib().p3dfft_gb300_set_pageable_direct(1 if on else 0)


def get_pageable_direct() -> int:
    """1 on, 0 off, -1 not supported by the device."""
    return int(lib().p3dfft_gb300_get_pageable_direct())


def set_stream(stream_ptr: int):
    lib().p3dfft_gb300_set_stream(ctypes.c_void_p(int(stream_ptr)))


def kernel_count() -> int:
    return int(lib().p3dfft_gb300_kernel_count())


def storage_shape(gdims, mo):
    """numpy shape (slowest dimension first) of a field of logical dims gdims stored with memory
    order mo (mo[d] = storage rank of logical dim d, 0 = stride-1)."""
    sd = [0, 0, 0]
    for i in range(3):
        sd[mo[i]] = gdims[i]
    return (sd[2], sd[1], sd[0])


def _ptr(a):
    """Returns (void pointer, keep-alive) for numpy arrays, torch tensors or int addresses."""
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise P3DFFTError("arrays must be C-contiguous")
        return ctypes.c_void_p(a.ctypes.data), a
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr()), a
    return ctypes.c_void_p(int(a)), None


class Transform3D:
    """transform3D<T1,T2>: the constructor plans (reference build/templ.C:91-420)."""

    def __init__(self, types, gdims1, mo1, gdims2, mo2, dcs1=-1, dcs2=-1):
        setup()
        self.types = tuple(int(t) for t in types)
        self.gdims1, self.mo1, self.dcs1 = tuple(gdims1), tuple(mo1), int(dcs1)
        self.gdims2, self.mo2, self.dcs2 = tuple(gdims2), tuple(mo2), int(dcs2)
        t = _i3(self.types)
        h = lib().p3dfft_gb300_plan3d(t, _i3(gdims1), _i3(mo1), self.dcs1, _i3(gdims2), _i3(mo2), self.dcs2)
        if h < 0:
            check(-1)
        self.handle = h
        a, b, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().p3dfft_gb300_plan3d_types(h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(p))
        self.dt1, self.dt2, self.prec = a.value, b.value, p.value

    def stages(self, executed=False):
        """The reference planner's stage list, or (executed=True) the schedule the executor runs."""
        buf = (ctypes.c_int * (16 * 8))()
        fn = lib().p3dfft_gb300_plan3d_exec_stages if executed else lib().p3dfft_gb300_plan3d_stages
        n = fn(self.handle, buf, 8)
        out = []
        for s in range(n):
            q = buf[16 * s:16 * s + 16]
            out.append(dict(type=q[0], dim=q[1], gdims1=tuple(q[2:5]), mo1=tuple(q[5:8]), dcs1=q[8],
                            gdims2=tuple(q[9:12]), mo2=tuple(q[12:15]), dcs2=q[15]))
        return out

    def in_dtype(self):
        return _np_dtype(self.dt1, self.prec)

    def out_dtype(self):
        return _np_dtype(self.dt2, self.prec)

    def in_shape(self):
        return storage_shape(self.gdims1, self.mo1)

    def out_shape(self):
        return storage_shape(self.gdims2, self.mo2)

    def exec(self, inp, out=None, OW=False, idir=-1):
        if out is None:
            out = np.empty(self.out_shape(), self.out_dtype())
        pi, _k1 = _ptr(inp)
        po, _k2 = _ptr(out)
        rc = lib().p3dfft_gb300_exec3d(self.handle, pi, po, int(idir), 1 if OW else 0)
        check(rc)
        return out

    def exec_deriv(self, inp, out=None, idir=0, OW=False):
        return self.exec(inp, out, OW=OW, idir=idir)

    _is1d = 0

    def autotune(self):
        check(lib().p3dfft_gb300_autotune(self.handle, self._is1d))
        return self.tuning()

    def tuning(self):
        """[(engine, talt, ms)] per stage; engine 0 = heuristic, 1 specialised, 2 register, 3 generic."""
        e, t, m = (ctypes.c_int * 8)(), (ctypes.c_int * 8)(), (ctypes.c_double * 8)()
        n = lib().p3dfft_gb300_plan_tuning(self.handle, self._is1d, e, t, m, 8)
        return [(e[i], t[i], m[i]) for i in range(n)]

    def set_engine(self, stage, engine, talt=0):
        check(lib().p3dfft_gb300_plan_set_engine(self.handle, self._is1d, int(stage), int(engine), int(talt)))

    def __del__(self):
        try:
            if getattr(self, "handle", -1) >= 0 and _lib is not None:
                _lib.p3dfft_gb300_destroy3d(self.handle)
        except Exception:
            pass


class TransPlan:
    """transplan<T1,T2>: one 1D transform with a local reorder (reference templ.C:900-1075)."""

    def __init__(self, type_id, gdims1, mo1, gdims2, mo2, dim, dcs1=-1, dcs2=-1):
        setup()
        self.type_id = int(type_id)
        self.gdims1, self.mo1 = tuple(gdims1), tuple(mo1)
        self.gdims2, self.mo2 = tuple(gdims2), tuple(mo2)
        self.dim = int(dim)
        h = lib().p3dfft_gb300_plan1d(self.type_id, _i3(gdims1), _i3(mo1), int(dcs1), _i3(gdims2), _i3(mo2),
                                      int(dcs2), self.dim)
        if h < 0:
            check(-1)
        self.handle = h

    def exec(self, inp, out, OW=False):
        pi, _k1 = _ptr(inp)
        po, _k2 = _ptr(out)
        check(lib().p3dfft_gb300_exec1d(self.handle, pi, po, 1 if OW else 0))
        return out

    _is1d = 1
    autotune = Transform3D.autotune
    tuning = Transform3D.tuning
    set_engine = Transform3D.set_engine

    def __del__(self):
        try:
            if getattr(self, "handle", -1) >= 0 and _lib is not None:
                _lib.p3dfft_gb300_destroy1d(self.handle)
        except Exception:
            pass


def compute_deriv(inp, out, gdims, mo, dcs, idir, prec=8):
    pi, _k1 = _ptr(inp)
    po, _k2 = _ptr(out)
    check(lib().p3dfft_gb300_compute_deriv(int(prec), pi, po, _i3(gdims), _i3(mo), int(dcs), int(idir)))
    return out


def _np_dtype(dt, prec):
    if dt == 2:
        return np.complex128 if prec == 8 else np.complex64
    return np.float64 if prec == 8 else np.float32


class DeviceArray:
    """A device allocation made by the library (no torch needed); frees on deletion."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = lib().p3dfft_gb300_device_alloc(self.nbytes)
        if not p:
            check(-1)
        self.ptr = int(p)

    def data_ptr(self):
        return self.ptr

    def upload(self, a: np.ndarray):
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        check(lib().p3dfft_gb300_memcpy_h2d(ctypes.c_void_p(self.ptr), ctypes.c_void_p(a.ctypes.data), a.nbytes))

    def download(self, a: np.ndarray):
        assert a.flags.c_contiguous and a.nbytes <= self.nbytes
        check(lib().p3dfft_gb300_memcpy_d2h(ctypes.c_void_p(a.ctypes.data), ctypes.c_void_p(self.ptr), a.nbytes))
        return a

    def __del__(self):
        try:
            if _lib is not None and self.ptr:
                _lib.p3dfft_gb300_device_free(ctypes.c_void_p(self.ptr))
        except Exception:
            pass


class PinnedArray:
    """numpy view over page-locked host memory allocated by the library."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        p = lib().p3dfft_gb300_host_alloc_pinned(n)
        if not p:
            check(-1)
        self.ptr = int(p)
        buf = (ctypes.c_char * n).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def __del__(self):
        try:
            if _lib is not None and self.ptr:
                self.array = None
                _lib.p3dfft_gb300_host_free_pinned(ctypes.c_void_p(self.ptr))
        except Exception:
            pass


class Batch:
    """Independent jobs run concurrently and replayed as one CUDA graph (p3dfft_gb300_batch_*).

    A job is an ordered list of steps (Transform3D, device input, device output, idir); the steps
    of one job run in order, different jobs run on concurrent branch streams."""

    def __init__(self, nbranches=0, graph=True, grouped=True):
        setup()
        h = lib().p3dfft_gb300_batch_create(int(nbranches))
        if h < 0:
            check(-1)
        self.handle = h
        self._keep = []
        if not graph:
            check(lib().p3dfft_gb300_batch_set_graph(h, 0))
        if grouped != 1:
            # False/0: branch streams; "list"/2: one work-list launch per kernel per level
            check(lib().p3dfft_gb300_batch_set_grouped(h, 2 if grouped in ("list", 2) else 0))

    def groups(self):
        return int(lib().p3dfft_gb300_batch_groups(self.handle))

    def add(self, job, plan, inp, out, idir=-1):
        pi, k1 = _ptr(inp)
        po, k2 = _ptr(out)
        self._keep += [plan, k1, k2]
        check(lib().p3dfft_gb300_batch_add(self.handle, int(job), plan.handle, pi, po, int(idir)))

    def exec(self):
        check(lib().p3dfft_gb300_batch_exec(self.handle))

    def kernels(self):
        return int(lib().p3dfft_gb300_batch_kernels(self.handle))

    def field_bytes(self):
        return float(lib().p3dfft_gb300_batch_field_bytes(self.handle))

    def __del__(self):
        try:
            if getattr(self, "handle", -1) >= 0 and _lib is not None:
                _lib.p3dfft_gb300_batch_destroy(self.handle)
        except Exception:
            pass


class Server:
    """Serving loop (p3dfft_gb300_server_*): jobs admitted under an HBM budget as they arrive,
    run concurrently on `nslots` streams."""

    def __init__(self, hbm_budget_bytes, nslots=8):
        setup()
        h = lib().p3dfft_gb300_server_create(int(hbm_budget_bytes), int(nslots))
        if h < 0:
            check(-1)
        self.handle = h
        self._keep = {}

    def clock(self):
        return float(lib().p3dfft_gb300_server_clock(self.handle))

    def submit(self, fwd, bwd, inp, out, idir=-1, arrival=-1.0):
        """Returns the job id.  `arrival` (server-clock seconds) >= 0 replays a trace."""
        pi, k1 = _ptr(inp)
        po, k2 = _ptr(out)
        j = lib().p3dfft_gb300_server_submit(self.handle, fwd.handle, bwd.handle, int(idir), pi, po, float(arrival))
        if j < 0:
            check(-1)
        self._keep[j] = (fwd, bwd, k1, k2)
        return j

    def wait(self, job, timeout=-1.0):
        rc = lib().p3dfft_gb300_server_wait(self.handle, int(job), float(timeout))
        if rc < 0:
            raise P3DFFTError(f"job {job} failed: {ERR_NAMES.get(-rc, -rc)}")
        return rc == 0

    def inject_alloc_failure(self, job):
        """Test hook: the job's device allocation fails at admission (it must still be waiting)."""
        check(lib().p3dfft_gb300_server_inject_alloc_failure(self.handle, int(job)))

    def drain(self):
        rc = lib().p3dfft_gb300_server_drain(self.handle)
        self._keep.clear()
        return rc

    def job_times(self, job):
        t = (ctypes.c_double * 3)()
        rc = lib().p3dfft_gb300_server_job_times(self.handle, int(job), t)
        return rc, (t[0], t[1], t[2])

    def stats(self):
        v = (ctypes.c_double * 8)()
        lib().p3dfft_gb300_server_stats(self.handle, v, 8)
        keys = ("completed", "failed", "admitted", "peak_hbm_bytes", "budget_bytes", "max_running",
                "host_launch_s", "host_release_s")
        return dict(zip(keys, [v[i] for i in range(8)]))

    def close(self):
        if getattr(self, "handle", -1) >= 0 and _lib is not None:
            _lib.p3dfft_gb300_server_destroy(self.handle)
            self.handle = -1

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_autotune(on: bool):
    lib().p3dfft_gb300_set_autotune(1 if on else 0)


def tune_cache_save(path):
    check(lib().p3dfft_gb300_tune_cache_save(os.fsencode(path)))


def tune_cache_load(path):
    n = lib().p3dfft_gb300_tune_cache_load(os.fsencode(path))
    if n < 0:
        check(-1)
    return n


def tune_cache_clear():
    lib().p3dfft_gb300_tune_cache_clear()
