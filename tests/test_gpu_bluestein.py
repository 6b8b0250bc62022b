"""GPU: lengths with a prime factor above 16 run on the Bluestein engine (a circular convolution
of a power-of-two length >= 2n-1 with a chirp; the reference leaves such lengths to FFTW's own
prime algorithms).  Compared with the CPU oracle (1e-12 relative L2 in FP64, 5e-6 in FP32) for
C2C, odd-length R2C / C2R and DCT/DST kinds whose extension length has a large prime factor, in
both tile orientations, and against the radix-pass engine it replaces."""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu

PRIMES = [17, 19, 31, 37, 61, 97, 139, 199, 257, 509, 1021]


def _run(p3d, oracle, tid_d, prec, dim, lin, lout, seed, engine=None):
    g1, g2 = [6, 5, 4], [6, 5, 4]
    g1[dim], g2[dim] = lin, lout
    mo1, mo2 = (0, 1, 2), ((0, 1, 2) if dim == 0 else (1, 0, 2))
    ti = oracle.type_info(tid_d)
    rng = np.random.default_rng(seed)
    shape = p3d.storage_shape(g1, mo1)
    x = rng.uniform(-1, 1, shape) + (1j * rng.uniform(-1, 1, shape) if ti["dt1"] == 2 else 0)
    ref = oracle.exec_stage(tid_d, dim, tuple(g1), mo1, tuple(g2), mo2, x)
    tid = tid_d if prec == 8 else tid_d - 1
    tp = p3d.TransPlan(tid, tuple(g1), mo1, tuple(g2), mo2, dim)
    if engine is not None:
        tp.set_engine(0, engine)
    if prec == 4:
        src = x.astype(np.complex64 if ti["dt1"] == 2 else np.float32)
        out = np.empty(ref.shape, np.complex64 if ti["dt2"] == 2 else np.float32)
    else:
        src, out = x, np.empty_like(ref)
    tp.exec(np.ascontiguousarray(src), out)
    return out, ref


@pytest.mark.parametrize("form", ["fp64_float_float", "fp64_native", "fp32"])
@pytest.mark.parametrize("dim", [0, 1])
def test_prime_c2c_and_odd_r2c_c2r(gpu, oracle, form, dim):
    p3d = gpu
    p3d.set_fp64_arith(0 if form == "fp64_native" else 1)
    prec = 4 if form == "fp32" else 8
    tol = 1e-12 if prec == 8 else 5e-6
    for n in PRIMES:
        for tid_d, lin, lout in ((9, n, n), (11, n, n), (5, n, n // 2 + 1), (7, n // 2 + 1, n)):
            if tid_d == 7:  # C2R from n//2+1 complex values to an odd n is rejected (reference sizes it 2(m-1))
                continue
            out, ref = _run(p3d, oracle, tid_d, prec, dim, lin, lout, seed=n)
            assert rel_l2(out, ref) < tol, (form, dim, n, tid_d, rel_l2(out, ref))


@pytest.mark.parametrize("prec", [8, 4])
def test_r2r_with_large_prime_extensions(gpu, oracle, prec):
    """DCT-I of n (extension 2(n-1)), DST-I (2(n+1)), DCT/DST II-IV (2n) with a prime > 16 in
    the extension length, real and complex data."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    cases = [("DCT1", 38), ("DST1", 36), ("DCT2", 37), ("DST2", 41), ("DCT3", 43), ("DST3", 29), ("DST4", 53),
             ("DCT1", 200)]
    for kind, n in cases:
        for data in ("REAL", "COMPLEX"):
            tid_d = p3d.TYPE_IDS[f"{kind}_{data}_D"]
            out, ref = _run(p3d, oracle, tid_d, prec, 0, n, n, seed=n)
            assert rel_l2(out, ref) < (1e-12 if prec == 8 else 5e-6), (kind, data, n, prec)


def test_bluestein_agrees_with_radix_passes(gpu, oracle):
    p3d = gpu
    p3d.set_fp64_arith(1)
    for n in (19, 139, 199):
        a, ref = _run(p3d, oracle, 9, 8, 0, n, n, seed=3, engine=4)  # Bluestein
        b, _ = _run(p3d, oracle, 9, 8, 0, n, n, seed=3, engine=3)    # radix passes, O(p^2) prime pass
        assert rel_l2(a, b) < 1e-13 and rel_l2(a, ref) < 1e-12


def test_uneven_sweep_grid_round_trip(gpu, oracle):
    """The reference's uneven sweep grid 58x139x199: R2C forward with d/dy, C2R backward."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd, gd2 = (58, 139, 199), (30, 139, 199)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    x = seeded_field((199, 139, 58), seed=58)
    y = f.exec(x)
    yo = oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x)
    assert rel_l2(y, yo) < 1e-12
    assert rel_l2(b.exec(y) / np.prod(gd), x) < 1e-12
    yd = f.exec_deriv(x, idir=1)
    ydo = oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x, idir=1)
    assert rel_l2(yd, ydo) < 1e-12
