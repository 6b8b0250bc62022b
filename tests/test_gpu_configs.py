"""GPU: the benchmark configurations at their full sizes, checked against the FP64 oracle.

Config 3 (mixed types and precision): a 384x256x257 field, x R2C, y C2C, z DCT-I (complex), the
field a sum of 8 seeded Chebyshev-Fourier modes plus 1e-3 uniform noise; run in FP64 (float-float
and native DFMA) and in FP32.  The relative L2 error against the FP64 oracle is stated for every
stage: each stage is run through the 1D transplan interface on the oracle's input for that stage.

Config 1 (64^3, plain FP64) and a 256^3 round trip are compared whole against the oracle.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu


def c3_field(gd, seed=3):
    """Sum of 8 Chebyshev-Fourier modes a_m cos(2 pi (kx x/Nx + ky y/Ny) + phi) T_n(cos(pi z/(Nz-1)))
    plus 1e-3 U[-1,1), in storage order (z, y, x) for memory order (0,1,2)."""
    nx, ny, nz = gd
    rng = np.random.default_rng(seed)
    x = np.arange(nx)[None, None, :] / nx
    y = np.arange(ny)[None, :, None] / ny
    theta = np.pi * np.arange(nz)[:, None, None] / (nz - 1)
    f = np.zeros((nz, ny, nx))
    for _ in range(8):
        a = rng.uniform(0.5, 1.5)
        kx, ky, n = rng.integers(0, 8), rng.integers(0, 8), rng.integers(0, 16)
        phi = rng.uniform(0, 2 * np.pi)
        f += a * np.cos(2 * np.pi * (kx * x + ky * y) + phi) * np.cos(n * theta)
    f += 1e-3 * rng.uniform(-1, 1, f.shape)
    return np.ascontiguousarray(f)


def _stage_errors(p3d, oracle, types_prec, types_d, gd, gd2, x, prec):
    op = oracle.OraclePlan(types_d, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    errs = []
    cur = x
    for st in op.stages():
        ref = oracle.exec_stage(st["type"], st["dim"], st["gdims1"], st["mo1"], st["gdims2"], st["mo2"], cur)
        tid = st["type"] if prec == 8 else st["type"] - 1  # _D -> _S type IDs are adjacent
        tp = p3d.TransPlan(tid, st["gdims1"], st["mo1"], st["gdims2"], st["mo2"], st["dim"], st["dcs1"], st["dcs2"])
        cdt = {8: (np.float64, np.complex128), 4: (np.float32, np.complex64)}[prec]
        ti = oracle.type_info(st["type"])
        src = np.ascontiguousarray(cur.astype(cdt[ti["dt1"] - 1]))
        out = np.empty(ref.shape, cdt[ti["dt2"] - 1])
        tp.exec(src, out)
        errs.append(rel_l2(out, ref))
        cur = ref
    return errs, op.exec(x)


@pytest.mark.parametrize("form", ["fp64_float_float", "fp64_native", "fp32"])
def test_config3_mixed_types_per_stage(gpu, oracle, form):
    p3d = gpu
    gd, gd2 = (384, 256, 257), (193, 256, 257)
    x = c3_field(gd)
    prec = 4 if form == "fp32" else 8
    p3d.set_fp64_arith(0 if form == "fp64_native" else 1)
    types_d = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.DCT1_COMPLEX_D]
    types = types_d if prec == 8 else [p3d.R2CFFT_S, p3d.CFFT_FORWARD_S, p3d.DCT1_COMPLEX_S]
    errs, y_oracle = _stage_errors(p3d, oracle, types, types_d, gd, gd2, x, prec)
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    y = f.exec(x.astype(np.float64 if prec == 8 else np.float32))
    e2e = rel_l2(y, y_oracle)
    print(f"config 3 {form}: per-stage rel L2 x={errs[0]:.2e} y={errs[1]:.2e} z={errs[2]:.2e}; 3D {e2e:.2e}")
    tol = 1e-12 if prec == 8 else 1e-6
    assert max(errs) < tol and e2e < tol


def test_config1_64cube_forward_and_round_trip(gpu, oracle):
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd, gd2 = (64, 64, 64), (33, 64, 64)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field((64, 64, 64), seed=64)
    y = f.exec(x)
    assert rel_l2(y, oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x)) < 1e-12
    assert rel_l2(b.exec(y) / 64 ** 3, x) < 1e-12


@pytest.mark.parametrize("arith", [1, 0])
def test_256cube_round_trip_with_derivative(gpu, oracle, arith):
    """A full 256^3 forward (fused d/dx) against the oracle, and the backward of the oracle
    spectrum, in both FP64 arithmetics."""
    p3d = gpu
    p3d.set_fp64_arith(arith)
    n = 256
    gd, gd2 = (n, n, n), (n // 2 + 1, n, n)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field((n, n, n), seed=256)
    yo = oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x, idir=0)
    assert rel_l2(f.exec_deriv(x, idir=0), yo) < 1e-12
    zo = oracle.OraclePlan(b.types, gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1).exec(yo)
    assert rel_l2(b.exec(yo), zo) < 1e-12


def test_executed_schedule_matches_reference_schedule(gpu, monkeypatch):
    """The executor's reordered schedule and the reference planner's stage list give the same
    transform (to rounding) for the headline plan shape, forward with d/dz and backward."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd, gd2 = (256, 128, 32), (129, 128, 32)  # planes of >= 16 Ki complex elements
    ft = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
    bt = [p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D]
    x = seeded_field((32, 128, 256), seed=11)
    out = {}
    for ref in ("1", "0"):
        monkeypatch.setenv("P3DFFT_GB300_REFERENCE_SCHEDULE", ref)
        f = p3d.Transform3D(ft, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
        b = p3d.Transform3D(bt, gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
        assert (f.stages(executed=True) == f.stages()) == (ref == "1")
        y = f.exec_deriv(x, idir=2)
        out[ref] = (y, b.exec(y))
    assert rel_l2(out["0"][0], out["1"][0]) < 1e-13
    assert rel_l2(out["0"][1], out["1"][1]) < 1e-13
