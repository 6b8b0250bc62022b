"""GPU: page-locked host arrays read by the first stage and written by the last stage directly
over NVLink-C2C (no staging copies).  Results must be bit-identical to the staged path and to
device-resident arrays: the same kernels run on the same values."""
import numpy as np
import pytest

from conftest import seeded_field

pytestmark = pytest.mark.gpu

CASES = [
    ("rcc", (64, 48, 40), (0, 1, 2), (1, 2, 0), 2),
    ("rcc", (40, 36, 30), (2, 0, 1), (0, 1, 2), 0),
    ("ccc", (32, 24, 20), (1, 0, 2), (2, 1, 0), -1),
    ("empty_mid", (48, 20, 18), (0, 1, 2), (2, 0, 1), -1),
]


def _plan(p3d, name, gd, mo1, mo2):
    types = {"rcc": ["R2CFFT_D", "CFFT_FORWARD_D", "CFFT_FORWARD_D"],
             "ccc": ["CFFT_FORWARD_D"] * 3,
             "empty_mid": ["R2CFFT_D", "EMPTY_TYPE_DOUBLE_COMPLEX", "CFFT_FORWARD_D"]}[name]
    ids = [p3d.TYPE_IDS[t] for t in types]
    gd2, dcs2 = list(gd), -1
    if types[0].startswith("R2C"):
        gd2[0], dcs2 = gd[0] // 2 + 1, 0
    return p3d.Transform3D(ids, gd, mo1, gd2, mo2, -1, dcs2)


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}-{c[3]}" for c in CASES])
def test_pinned_direct_equals_staged_and_device(gpu, case):
    p3d = gpu
    p3d.set_fp64_arith(1)
    name, gd, mo1, mo2, idir = case
    f = _plan(p3d, name, gd, mo1, mo2)
    dt = f.in_dtype()
    x = seeded_field(f.in_shape(), seed=sum(gd), dtype=dt)
    hin = p3d.PinnedArray(x.shape, dt)
    hin.array[...] = x
    outs = {}
    for direct in (True, False):
        p3d.set_host_direct(direct)
        hout = p3d.PinnedArray(f.out_shape(), f.out_dtype())
        hout.array[...] = 0
        f.exec(hin.array, hout.array, idir=idir)
        outs[direct] = hout.array.copy()
    p3d.set_host_direct(True)
    d_in, d_out = p3d.DeviceArray(x.nbytes), p3d.DeviceArray(outs[True].nbytes)
    d_in.upload(x)
    f.exec(d_in, d_out, idir=idir)
    y_dev = d_out.download(np.empty_like(outs[True]))
    assert np.array_equal(outs[True], outs[False])
    assert np.array_equal(outs[True], y_dev)
    assert np.array_equal(hin.array, x)  # the input is not modified


def test_pinned_in_place_is_staged(gpu):
    """in == out on page-locked memory: staged through HBM (the kernels never read and write the
    same host array), result equal to the out-of-place call."""
    p3d = gpu
    gd = (16, 12, 10)
    f = _plan(p3d, "ccc", gd, (0, 1, 2), (0, 1, 2))
    x = seeded_field(f.in_shape(), seed=3, dtype=np.complex128)
    buf = p3d.PinnedArray(x.shape, np.complex128)
    buf.array[...] = x
    ref = f.exec(x)
    f.exec(buf.array, buf.array)
    assert np.array_equal(buf.array, ref)


def test_large_staged_field_overlapped_in_slabs(gpu, oracle):
    """A pageable 256x256x160 FP64 field (over the 32 MB slab threshold): its copies are overlapped
    with the first and last stages slab by slab; the result equals the device-resident one."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd = (256, 256, 160)
    f = _plan(p3d, "rcc", gd, (0, 1, 2), (1, 2, 0))
    gd2 = (129, 256, 160)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field(f.in_shape(), seed=5)
    k0 = p3d.kernel_count()
    y = f.exec(x)  # pageable numpy in and out: staged
    assert p3d.kernel_count() - k0 > 3  # the first stage ran in slabs
    z = b.exec(y)
    d_in, d_s, d_out = p3d.DeviceArray(x.nbytes), p3d.DeviceArray(y.nbytes), p3d.DeviceArray(x.nbytes)
    d_in.upload(x)
    f.exec(d_in, d_s)
    b.exec(d_s, d_out)
    assert np.array_equal(y, d_s.download(np.empty_like(y)))
    assert np.array_equal(z, d_out.download(np.empty_like(z)))


# (the (2,0,1) input layout has the x dim slowest: the x stage cannot be cut into slabs there,
# so that plan runs stage after stage either way)
@pytest.mark.parametrize("prec,mo1,mo2,sliced", [(8, (0, 1, 2), (1, 2, 0), True), (8, (2, 0, 1), (0, 1, 2), False),
                                                 (4, (0, 1, 2), (1, 2, 0), True)])
def test_pinned_host_stages_pipelined_equal_device(gpu, prec, mo1, mo2, sliced):
    """Page-locked host input and output of a 3D round trip (fields over the 32 MB threshold,
    d/dz fused), read / written directly by the kernels, or staged through HBM by per-slab
    copies with the first two / last two stages pipelined behind them slab by slab (or, with
    pipelining off, the first / last stage alone), or read / written directly by a first / last
    stage capped at a few persistent CTAs with its neighbour stage beside it slab by slab: every
    variant bit-identical to device-resident arrays."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd = (256, 256, 160) if prec == 8 else (256, 256, 192)
    gd2 = (129, gd[1], gd[2])
    S = "D" if prec == 8 else "S"
    f = p3d.Transform3D([p3d.TYPE_IDS[f"R2CFFT_{S}"], p3d.TYPE_IDS[f"CFFT_FORWARD_{S}"],
                         p3d.TYPE_IDS[f"CFFT_FORWARD_{S}"]], gd, mo1, gd2, mo2, -1, 0)
    b = p3d.Transform3D([p3d.TYPE_IDS[f"C2RFFT_{S}"], p3d.TYPE_IDS[f"CFFT_BACKWARD_{S}"],
                         p3d.TYPE_IDS[f"CFFT_BACKWARD_{S}"]], gd2, mo2, gd, mo1, 0, -1)
    rdt = np.float64 if prec == 8 else np.float32
    x = seeded_field(f.in_shape(), seed=11, dtype=rdt)
    hin = p3d.PinnedArray(x.shape, rdt)
    hin.array[...] = x
    d_s = p3d.DeviceArray(int(np.prod(f.out_shape())) * np.dtype(f.out_dtype()).itemsize)
    res = {}
    try:
        p3d.set_link_ctas(0)  # direct host access stage after stage, first
        for direct in (True, False):
            p3d.set_host_direct(direct)
            for pipe in (True, False):
                p3d.set_host_pipeline(pipe)
                hout = p3d.PinnedArray(x.shape, rdt)
                hout.array[...] = 0
                k0 = p3d.kernel_count()
                f.exec(hin.array, d_s, idir=2)
                spec = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
                b.exec(d_s, hout.array)
                res[direct, pipe] = (spec, hout.array.copy(), p3d.kernel_count() - k0)
        p3d.set_host_direct(True)
        p3d.set_host_pipeline(True)
        for cap in (37, 152, -1):  # persistent link-stage CTAs (37: many tiles per CTA; -1 default)
            p3d.set_link_ctas(cap)
            hout = p3d.PinnedArray(x.shape, rdt)
            hout.array[...] = 0
            k0 = p3d.kernel_count()
            f.exec(hin.array, d_s, idir=2)
            spec = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
            b.exec(d_s, hout.array)
            res["link", cap] = (spec, hout.array.copy(), p3d.kernel_count() - k0)
    finally:
        p3d.set_link_ctas(-1)
        p3d.set_host_pipeline(True)
        p3d.set_host_direct(True)
    assert res[True, True][2] == res[True, False][2]  # direct host access: stage after stage
    assert res["link", 37][2] > res[True, True][2]  # the linked stage pairs ran in slabs
    if sliced:  # staged: the stage pairs (pipelining on) or the end stages (off) ran in slabs
        assert res[False, True][2] > res[False, False][2] > res[True, True][2]
    else:
        assert res[False, True][2] == res[False, False][2] == res[True, True][2]
    d_in, d_out = p3d.DeviceArray(x.nbytes), p3d.DeviceArray(x.nbytes)
    d_in.upload(x)
    f.exec(d_in, d_s, idir=2)
    spec_dev = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
    b.exec(d_s, d_out)
    y_dev = d_out.download(np.empty_like(x))
    for key, (spec, y, _) in res.items():
        assert np.array_equal(spec, spec_dev), key
        assert np.array_equal(y, y_dev), key
    assert np.array_equal(hin.array, x)


@pytest.mark.parametrize("arith,gd,mo1,mo2", [(1, (512, 128, 70), (0, 1, 2), (1, 2, 0)),
                                              (0, (256, 256, 136), (0, 1, 2), (1, 2, 0)),
                                              (1, (512, 96, 90), (1, 0, 2), (2, 1, 0))])
def test_link_pipelined_ragged_slabs_and_native_fp64(gpu, arith, gd, mo1, mo2):
    """Direct host input / output with the link stages on capped persistent grids beside their
    neighbour stages: slab dims of 70 and 90 planes (large slabs and a thin one, ragged),
    native FP64 arithmetic (IEEE intermediates), and another memory-order pair; each equal bit for
    bit to the same round trip stage after stage (cap 0) and to device-resident arrays."""
    p3d = gpu
    p3d.set_fp64_arith(arith)
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    f = p3d.Transform3D([p3d.TYPE_IDS["R2CFFT_D"], p3d.TYPE_IDS["CFFT_FORWARD_D"],
                         p3d.TYPE_IDS["CFFT_FORWARD_D"]], gd, mo1, gd2, mo2, -1, 0)
    b = p3d.Transform3D([p3d.TYPE_IDS["C2RFFT_D"], p3d.TYPE_IDS["CFFT_BACKWARD_D"],
                         p3d.TYPE_IDS["CFFT_BACKWARD_D"]], gd2, mo2, gd, mo1, 0, -1)
    x = seeded_field(f.in_shape(), seed=sum(gd) + arith)
    hin = p3d.PinnedArray(x.shape, np.float64)
    hin.array[...] = x
    d_s = p3d.DeviceArray(int(np.prod(f.out_shape())) * 16)
    res = {}
    try:
        for cap in (0, -1, 61):
            p3d.set_link_ctas(cap)
            hout = p3d.PinnedArray(x.shape, np.float64)
            hout.array[...] = 0
            k0 = p3d.kernel_count()
            f.exec(hin.array, d_s)
            spec = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
            b.exec(d_s, hout.array)
            res[cap] = (spec, hout.array.copy(), p3d.kernel_count() - k0)
    finally:
        p3d.set_link_ctas(-1)
        p3d.set_fp64_arith(1)
    assert res[-1][2] > res[0][2] and res[61][2] == res[-1][2]  # slab launches in the linked pairs
    d_in, d_out = p3d.DeviceArray(x.nbytes), p3d.DeviceArray(x.nbytes)
    d_in.upload(x)
    p3d.set_fp64_arith(arith)
    try:
        f.exec(d_in, d_s)
        spec_dev = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
        b.exec(d_s, d_out)
        y_dev = d_out.download(np.empty_like(x))
    finally:
        p3d.set_fp64_arith(1)
    for cap, (spec, y, _) in res.items():
        assert np.array_equal(spec, spec_dev), cap
        assert np.array_equal(y, y_dev), cap
    rel = np.linalg.norm(y_dev / np.prod(gd) - x) / np.linalg.norm(x)
    assert rel < 1e-13, rel


@pytest.mark.parametrize("side", ["in", "out"])
def test_link_pipeline_one_side_direct(gpu, side):
    """One host array read (or written) directly with its link stage pipelined beside the
    neighbour stage, the other staged through HBM with per-slab copies (FP32, 50 MB fields): the
    result equal bit for bit to device-resident arrays."""
    p3d = gpu
    gd = (512, 160, 160)
    gd2 = (257, gd[1], gd[2])
    f = p3d.Transform3D([p3d.TYPE_IDS["R2CFFT_S"], p3d.TYPE_IDS["CFFT_FORWARD_S"],
                         p3d.TYPE_IDS["CFFT_FORWARD_S"]], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.TYPE_IDS["C2RFFT_S"], p3d.TYPE_IDS["CFFT_BACKWARD_S"],
                         p3d.TYPE_IDS["CFFT_BACKWARD_S"]], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field(f.in_shape(), seed=77, dtype=np.float32)
    hin = p3d.PinnedArray(x.shape, np.float32)
    hin.array[...] = x
    hout = p3d.PinnedArray(x.shape, np.float32)
    d_s = p3d.DeviceArray(int(np.prod(f.out_shape())) * 8)
    try:
        p3d.set_host_direct(side)
        f.exec(hin.array, d_s, idir=2)
        spec = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
        b.exec(d_s, hout.array)
    finally:
        p3d.set_host_direct(True)
    d_in, d_out = p3d.DeviceArray(x.nbytes), p3d.DeviceArray(x.nbytes)
    d_in.upload(x)
    f.exec(d_in, d_s, idir=2)
    assert np.array_equal(spec, d_s.download(np.empty(f.out_shape(), f.out_dtype())))
    b.exec(d_s, d_out)
    assert np.array_equal(hout.array, d_out.download(np.empty_like(x)))


@pytest.mark.parametrize("prec,gd,mo1,mo2", [(8, (64, 48, 40), (0, 1, 2), (1, 2, 0)),
                                              (8, (512, 128, 80), (0, 1, 2), (1, 2, 0)),
                                              (4, (512, 160, 128), (2, 0, 1), (0, 1, 2))])
def test_pageable_arrays_in_place_equal_device(gpu, prec, gd, mo1, mo2):
    """Pageable host arrays (plain numpy memory; the output's pages untouched before the call) read
    and written in place by the end stages through the host's page tables, the larger fields with
    the link pipeline: equal bit for bit to device-resident arrays and to the staged path."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    S = "D" if prec == 8 else "S"
    f = p3d.Transform3D([p3d.TYPE_IDS[f"R2CFFT_{S}"], p3d.TYPE_IDS[f"CFFT_FORWARD_{S}"],
                         p3d.TYPE_IDS[f"CFFT_FORWARD_{S}"]], gd, mo1, gd2, mo2, -1, 0)
    b = p3d.Transform3D([p3d.TYPE_IDS[f"C2RFFT_{S}"], p3d.TYPE_IDS[f"CFFT_BACKWARD_{S}"],
                         p3d.TYPE_IDS[f"CFFT_BACKWARD_{S}"]], gd2, mo2, gd, mo1, 0, -1)
    x = seeded_field(f.in_shape(), seed=sum(gd) + 5, dtype=np.float64 if prec == 8 else np.float32)
    d_s = p3d.DeviceArray(int(np.prod(f.out_shape())) * 2 * prec)
    res = {}
    try:
        for direct in (False, True):
            p3d.set_pageable_direct(direct)
            if direct and p3d.get_pageable_direct() != 1:
                pytest.skip("the device does not access pageable memory through the host's page tables")
            y = np.empty_like(x)
            f.exec(x, d_s, idir=2)
            spec = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
            b.exec(d_s, y)
            res[direct] = (spec, y)
    finally:
        p3d.set_pageable_direct(False)
    d_in, d_out = p3d.DeviceArray(x.nbytes), p3d.DeviceArray(x.nbytes)
    d_in.upload(x)
    f.exec(d_in, d_s, idir=2)
    spec_dev = d_s.download(np.empty(f.out_shape(), f.out_dtype()))
    b.exec(d_s, d_out)
    y_dev = d_out.download(np.empty_like(x))
    for direct, (spec, y) in res.items():
        assert np.array_equal(spec, spec_dev), direct
        assert np.array_equal(y, y_dev), direct
