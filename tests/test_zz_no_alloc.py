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
