"""GPU: FP32 stages whose tile input is fetched by TMA (a tensor map over the input and
cp.async.bulk.tensor into shared memory) instead of per-thread global loads.

The same values reach the same butterflies either way, so results are bit-identical to the
per-thread-load kernels, and within 1e-6 relative L2 of the FP64 oracle.  The TMA path must
actually run (launch counter), also for a partial last tile and for the 3D round trip's
line-contiguous stages.  Its bounded wait is tested by an injected stall: every tile's wait runs
out (20 ms), the status word is set, and the context stays usable.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu

C2C_LENGTHS = [32, 64, 128, 256, 384, 512, 1024, 2048]
R2C_LENGTHS = [64, 128, 256, 512, 1024, 2048]  # real lengths: FFT lengths 32 .. 1024


def _line_plan(p3d, kind, n, lines):
    g1 = [n, lines[0], lines[1]]
    g2 = list(g1)
    tid = {"c2c": p3d.CFFT_FORWARD_S, "r2c": p3d.R2CFFT_S}[kind]
    if kind == "r2c":
        g2[0] = n // 2 + 1
    return p3d.TransPlan(tid, tuple(g1), (0, 1, 2), tuple(g2), (0, 1, 2), 0), g1, g2


def _run(p3d, plan, x, g2, dt, tma):
    p3d.set_fp32_tma(tma)
    y = np.empty(p3d.storage_shape(g2, (0, 1, 2)), dt)
    c0 = p3d.tma_launch_count()
    plan.exec(np.ascontiguousarray(x), y)
    return y, p3d.tma_launch_count() - c0


@pytest.mark.parametrize("kind,n", [("c2c", n) for n in C2C_LENGTHS] + [("r2c", n) for n in R2C_LENGTHS])
def test_tma_lines_bit_identical_and_oracle(gpu, oracle, kind, n):
    p3d = gpu
    lines = (24, 7)  # 168 lines: a partial last tile for most tile sizes
    plan, g1, g2 = _line_plan(p3d, kind, n, lines)
    cplx = kind == "c2c"
    x = seeded_field(p3d.storage_shape(g1, (0, 1, 2)), seed=n, dtype=np.complex64 if cplx else np.float32)
    try:
        y_t, used = _run(p3d, plan, x, g2, np.complex64, True)
        y_l, unused = _run(p3d, plan, x, g2, np.complex64, False)
    finally:
        p3d.set_fp32_tma(True)
    assert used == 1 and unused == 0
    assert np.array_equal(y_t, y_l)
    tid_d = p3d.CFFT_FORWARD_D if cplx else p3d.R2CFFT_D
    ref = oracle.exec_stage(tid_d, 0, tuple(g1), (0, 1, 2), tuple(g2), (0, 1, 2),
                            x.astype(np.complex128 if cplx else np.float64))
    assert rel_l2(y_t, ref) < 1e-6
    assert p3d.device_status() == 0


def test_tma_round_trip_3d(gpu, oracle):
    """A 128^3 FP32 R2C/C2C/C2C forward with d/dz and its backward, memory orders
    (0,1,2) <-> (1,2,0): the x R2C and the backward stages with contiguous lines run TMA-staged;
    results equal the per-thread-load kernels bit for bit."""
    p3d = gpu
    gd, gd2 = (128, 128, 128), (65, 128, 128)
    f = p3d.Transform3D([p3d.R2CFFT_S, p3d.CFFT_FORWARD_S, p3d.CFFT_FORWARD_S], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_S, p3d.CFFT_BACKWARD_S, p3d.CFFT_BACKWARD_S], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field(f.in_shape(), seed=7, dtype=np.float32)
    out = {}
    try:
        for tma in (True, False):
            p3d.set_fp32_tma(tma)
            c0 = p3d.tma_launch_count()
            s = f.exec(x, idir=2)
            y = b.exec(s)
            out[tma] = (s, y, p3d.tma_launch_count() - c0)
    finally:
        p3d.set_fp32_tma(True)
    assert out[True][2] >= 2 and out[False][2] == 0
    assert np.array_equal(out[True][0], out[False][0])
    assert np.array_equal(out[True][1], out[False][1])
    assert p3d.device_status() == 0


def test_tma_wait_runs_out_sets_status(gpu):
    """An injected stall (the tile's barrier expects 16 bytes that never arrive): every tile's
    wait gives up after 20 ms and sets the status word; the call returns, the status reads 1
    and clears, and the next transform is correct."""
    p3d = gpu
    plan, g1, g2 = _line_plan(p3d, "c2c", 256, (8, 2))  # 16 lines: two tiles
    x = seeded_field(p3d.storage_shape(g1, (0, 1, 2)), seed=3, dtype=np.complex64)
    p3d.set_fp32_tma(True)
    assert p3d.device_status() == 0
    p3d.inject_tma_stall()
    _run(p3d, plan, x, g2, np.complex64, True)
    assert p3d.device_status() == 1
    assert p3d.device_status() == 0  # cleared by the read
    y, used = _run(p3d, plan, x, g2, np.complex64, True)
    y_l, _ = _run(p3d, plan, x, g2, np.complex64, False)
    p3d.set_fp32_tma(True)
    assert used == 1 and np.array_equal(y, y_l)
    assert p3d.device_status() == 0


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024])
def test_tma_tile_dim_contiguous_c2c(gpu, oracle, n):
    """C2C lines along dim 1 of a (0,1,2) layout: the tile dim (dim 0, 64 points) is contiguous, so
    each tile arrives as rows of its lines' points (TMA mode 2); bit-identical to per-thread loads,
    and a tile dim that is not a multiple of the tile's lines (63) takes the per-thread loads."""
    p3d = gpu
    for dt, expect in ((64, 1), (63, 0)):
        g = (dt, n, 3)
        tp = p3d.TransPlan(p3d.CFFT_FORWARD_S, g, (0, 1, 2), g, (0, 1, 2), 1)
        x = seeded_field(p3d.storage_shape(g, (0, 1, 2)), seed=n + dt, dtype=np.complex64)
        out = {}
        try:
            for tma in (True, False):
                p3d.set_fp32_tma(tma)
                y = np.empty(p3d.storage_shape(g, (0, 1, 2)), np.complex64)
                c0 = p3d.tma_launch_count()
                tp.exec(np.ascontiguousarray(x), y)
                out[tma] = (y, p3d.tma_launch_count() - c0)
        finally:
            p3d.set_fp32_tma(True)
        assert out[True][1] == expect and out[False][1] == 0, (n, dt, out[True][1])
        assert np.array_equal(out[True][0], out[False][0]), (n, dt)
        ref = oracle.exec_stage(p3d.CFFT_FORWARD_D, 1, g, (0, 1, 2), g, (0, 1, 2), x.astype(np.complex128))
        assert rel_l2(out[True][0], ref) < 1e-6
    assert p3d.device_status() == 0
