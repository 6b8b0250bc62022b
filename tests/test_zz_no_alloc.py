"""The allocation-free 3D entry point, p3dfft_gb300_exec3d_noalloc.

Callers that cannot call cudaMalloc -- applications whose device memory is all owned by their own
allocator, real-time loops that may not take cudaMalloc's implicit device synchronisation,
plugin hosts that forbid device allocations -- run a 3D plan through this entry point, which
keeps the intermediate fields and twiddle tables in a static device array of the library instead
of allocating them.  These tests call it through the C ABI and check it against the regular
entry point, p3dfft_gb300_exec3d, within the FP64 parity tolerance used by the other GPU tests,
on two calls in a row (the static array keeps the previous call's contents).

The file name sorts last so that a run stopping at its first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _vp(x):
    return ctypes.c_void_p(int(x))


def test_noalloc_matches_exec3d_two_calls(gpu):
    p3d = gpu
    L = p3d.lib()
    gd, gd2 = (64, 48, 40), (33, 48, 40)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=31)
    s_r, s_c = x.nbytes, 16 * int(np.prod(gd2))
    d_in, d_spec_ref, d_spec = p3d.DeviceArray(s_r), p3d.DeviceArray(s_c), p3d.DeviceArray(s_c)
    d_out_ref, d_out = p3d.DeviceArray(s_r), p3d.DeviceArray(s_r)
    d_in.upload(x)

    # regular entry point: forward with fused d/dy, then backward
    p3d.check(L.p3dfft_gb300_exec3d(f.handle, _vp(d_in.ptr), _vp(d_spec_ref.ptr), 1, 0))
    p3d.check(L.p3dfft_gb300_exec3d(b.handle, _vp(d_spec_ref.ptr), _vp(d_out_ref.ptr), -1, 0))
    spec_ref = d_spec_ref.download(np.empty(p3d.storage_shape(gd2, (1, 2, 0)), np.complex128))
    out_ref = d_out_ref.download(np.empty(p3d.storage_shape(gd, (0, 1, 2)), np.float64))

    for call in range(2):
        p3d.check(L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in.ptr), _vp(d_spec.ptr), 1))
        p3d.check(L.p3dfft_gb300_exec3d_noalloc(b.handle, _vp(d_spec.ptr), _vp(d_out.ptr), -1))
        spec = d_spec.download(np.empty_like(spec_ref))
        out = d_out.download(np.empty_like(out_ref))
        assert rel_l2(spec, spec_ref) < TOL64, call
        assert rel_l2(out, out_ref) < TOL64, call


def test_noalloc_rejects_host_pointers_and_oversize(gpu):
    p3d = gpu
    L = p3d.lib()
    gd, gd2 = (16, 8, 8), (9, 8, 8)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    x = np.zeros(p3d.storage_shape(gd, (0, 1, 2)))
    y = np.zeros(p3d.storage_shape(gd2, (1, 2, 0)), np.complex128)
    rc = L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(x.ctypes.data), _vp(y.ctypes.data), -1)
    assert rc == 1  # P3DFFT_ERR_BAD_ARG: device memory only
    L.p3dfft_clear_error()

    limit = L.p3dfft_gb300_noalloc_max_field_bytes()
    big = (512, 512, 64)  # intermediate spectrum 257*512*64*16 B, above the static limit
    big2 = (257, 512, 64)
    assert 16 * int(np.prod(big2)) > limit
    g = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], big, (0, 1, 2), big2, (1, 2, 0), -1, 0)
    d_in, d_out = p3d.DeviceArray(8 * int(np.prod(big))), p3d.DeviceArray(16 * int(np.prod(big2)))
    rc = L.p3dfft_gb300_exec3d_noalloc(g.handle, _vp(d_in.ptr), _vp(d_out.ptr), -1)
    assert rc == 5  # P3DFFT_ERR_TOO_LARGE
    L.p3dfft_clear_error()


def _device(p3d, a):
    d = p3d.DeviceArray(a.nbytes)
    d.upload(a)
    return d


def _run_both(p3d, f, x, out_shape, out_dtype, idir, offset=0):
    """Runs plan f on x through exec3d and through exec3d_noalloc (device buffers, optionally
    offset by `offset` bytes); returns both outputs."""
    L = p3d.lib()
    nb_out = int(np.prod(out_shape)) * np.dtype(out_dtype).itemsize
    d_in = p3d.DeviceArray(x.nbytes + 64)
    d_in_ptr = d_in.ptr + offset
    L.p3dfft_gb300_memcpy_h2d(_vp(d_in_ptr), _vp(x.ctypes.data), x.nbytes)
    d_a, d_b = p3d.DeviceArray(nb_out + 64), p3d.DeviceArray(nb_out + 64)
    p3d.check(L.p3dfft_gb300_exec3d(f.handle, _vp(d_in_ptr), _vp(d_a.ptr + offset), idir, 0))
    p3d.check(L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in_ptr), _vp(d_b.ptr + offset), idir))
    a, b = np.empty(out_shape, out_dtype), np.empty(out_shape, out_dtype)
    L.p3dfft_gb300_memcpy_d2h(_vp(a.ctypes.data), _vp(d_a.ptr + offset), nb_out)
    L.p3dfft_gb300_memcpy_d2h(_vp(b.ctypes.data), _vp(d_b.ptr + offset), nb_out)
    return a, b


def test_noalloc_matches_oracle(gpu, oracle):
    """Forward R2C / C2C / C2C with the fused d/dz derivative, checked against the CPU oracle."""
    p3d = gpu
    gd, gd2 = (48, 40, 36), (25, 40, 36)
    types = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=37)
    d_in = _device(p3d, x)
    d_out = p3d.DeviceArray(16 * int(np.prod(gd2)))
    p3d.check(p3d.lib().p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in.ptr), _vp(d_out.ptr), 2))
    y = d_out.download(np.empty(p3d.storage_shape(gd2, (1, 2, 0)), np.complex128))
    yo = oracle.OraclePlan(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x, idir=2)
    assert rel_l2(y, yo) < TOL64


def test_noalloc_makes_no_device_allocation(gpu):
    """Device free memory is unchanged across the first noalloc call of a fresh plan (after one
    call of another plan, which resolves the static array)."""
    torch = pytest.importorskip("torch")
    p3d = gpu
    L = p3d.lib()
    gd, gd2 = (64, 64, 64), (33, 64, 64)
    types = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
    warm = p3d.Transform3D(types, (16, 8, 8), (0, 1, 2), (9, 8, 8), (1, 2, 0), -1, 0)
    d_wi, d_wo = p3d.DeviceArray(8 * 16 * 64), p3d.DeviceArray(16 * 9 * 64)
    p3d.check(L.p3dfft_gb300_exec3d_noalloc(warm.handle, _vp(d_wi.ptr), _vp(d_wo.ptr), -1))
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    d_in = _device(p3d, seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=41))
    d_out = p3d.DeviceArray(16 * int(np.prod(gd2)))
    p3d.check(L.p3dfft_gb300_synchronize())
    free0, _ = torch.cuda.mem_get_info()
    p3d.check(L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in.ptr), _vp(d_out.ptr), 2))
    p3d.check(L.p3dfft_gb300_synchronize())
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_derivative_on_dct1_stage(gpu):
    """The derivative stage is a complex DCT-I, whose kernel (and table format) differs from the
    same stage without the derivative: the tables must be those of the launched kernel."""
    p3d = gpu
    gd = (24, 20, 17)
    gd2 = (13, 20, 17)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.DCT1_COMPLEX_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=43)
    for idir in (2, 0):
        a, b = _run_both(p3d, f, x, p3d.storage_shape(gd2, (1, 2, 0)), np.complex128, idir)
        assert rel_l2(b, a) < TOL64, idir


def test_noalloc_unaligned_real_r2r(gpu):
    """Real DCT-II / DST-II / DCT-III plan on buffers 8 bytes off a 16-byte boundary: the
    kernel choice (and table format) depends on the alignment."""
    p3d = gpu
    gd = (20, 16, 12)
    f = p3d.Transform3D([p3d.DCT2_REAL_D, p3d.DST2_REAL_D, p3d.DCT3_REAL_D], gd, (0, 1, 2), gd, (1, 2, 0))
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=47)
    for off in (0, 8):
        a, b = _run_both(p3d, f, x, p3d.storage_shape(gd, (1, 2, 0)), np.float64, -1, offset=off)
        assert rel_l2(b, a) < TOL64, off


def test_noalloc_autotuned_plan(gpu):
    """With the autotuner on, a stage may be tuned to an engine that needs the library's cached
    tables (Bluestein for a length with a prime factor above 16); that stage runs the heuristic
    engine here and the result still matches exec3d."""
    p3d = gpu
    L = p3d.lib()
    gd, gd2 = (34, 38, 32), (18, 38, 32)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    f.autotune()
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=53)
    a, b = _run_both(p3d, f, x, p3d.storage_shape(gd2, (1, 2, 0)), np.complex128, 1)
    assert rel_l2(b, a) < TOL64
    L.p3dfft_clear_error()


def test_noalloc_largest_tables(gpu):
    """The largest twiddle tables a plan within the scratch limit can need: a 3072 x 3072 x 1 real
    DCT-II / DST-II / DCT-II plan (two lines of 3072 points with their pre/post-twiddle tables,
    983,552 bytes of the 1 MiB table region, each table starting on a 256-byte boundary)."""
    p3d = gpu
    gd = (3072, 3072, 1)
    f = p3d.Transform3D([p3d.DCT2_REAL_D, p3d.DST2_REAL_D, p3d.DCT2_REAL_D], gd, (0, 1, 2), gd, (1, 0, 2))
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=59)
    a, b = _run_both(p3d, f, x, p3d.storage_shape(gd, (1, 0, 2)), np.float64, -1)
    assert rel_l2(b, a) < TOL64


def test_noalloc_refuses_a_capturing_stream(gpu):
    """Tables are staged through a static host array that the next call overwrites, so the entry
    point refuses to run while its stream is being captured (nothing is enqueued)."""
    torch = pytest.importorskip("torch")
    p3d = gpu
    L = p3d.lib()
    gd, gd2 = (16, 8, 8), (9, 8, 8)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    d_in, d_out = p3d.DeviceArray(8 * 16 * 64), p3d.DeviceArray(16 * 9 * 64)
    p3d.check(L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in.ptr), _vp(d_out.ptr), -1))
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    p3d.set_stream(s.cuda_stream)
    try:
        with torch.cuda.graph(g, stream=s):
            rc = L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in.ptr), _vp(d_out.ptr), -1)
    finally:
        p3d.set_stream(0)
    assert rc == 2  # P3DFFT_ERR_UNSUPPORTED
    L.p3dfft_clear_error()
    p3d.check(L.p3dfft_gb300_exec3d_noalloc(f.handle, _vp(d_in.ptr), _vp(d_out.ptr), -1))
