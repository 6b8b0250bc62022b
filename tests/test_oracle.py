"""CPU: pins the oracle (oracle/p3d_oracle.c) before it is trusted as the checker.

1. FFTW transform definitions: against an O(n^2) long-double direct DFT and against scipy.fft
   (pocketfft, whose unnormalised DCT/DST types 1-4 are FFTW's REDFT/RODFT kinds).
2. The analytic known answers of the reference's own sample programs (sample/C++/test3D_r2c.C,
   test_deriv.C, test1D_cos.C, test1D_sin.C), through the oracle's 3D / stage executor.
3. The committed golden fixtures in tests/golden/ (generated by tests/golden/make_golden.py).
"""
import itertools
import os

import numpy as np
import pytest

from conftest import rel_l2, seeded_field

scipy_fft = pytest.importorskip("scipy.fft")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 12, 16, 17, 31, 64])
def test_fft_against_long_double_direct(oracle, n):
    x = seeded_field((n,), seed=n, dtype=np.complex128)
    for sign in (-1, 1):
        assert rel_l2(oracle.dft_c2c(x, sign), oracle.dft_c2c(x, sign, direct=True)) < 5e-16 * max(1, np.log2(n))


@pytest.mark.parametrize("n", [2, 3, 4, 7, 9, 16, 25, 64, 97, 129, 257, 384, 512])
def test_transforms_against_scipy(oracle, n):
    x = seeded_field((n,), seed=100 + n)
    z = seeded_field((n,), seed=200 + n, dtype=np.complex128)
    assert rel_l2(oracle.dft_c2c(z, -1), scipy_fft.fft(z)) < 1e-15
    assert rel_l2(oracle.dft_c2c(z, +1), scipy_fft.ifft(z) * n) < 1e-15
    assert rel_l2(oracle.dft_r2c(x), scipy_fft.rfft(x)) < 1e-15
    X = scipy_fft.rfft(x)
    assert rel_l2(oracle.dft_c2r(X, n), scipy_fft.irfft(X, n) * n) < 1e-15
    kinds = [(oracle.REDFT00, "dct", 1), (oracle.REDFT10, "dct", 2), (oracle.REDFT01, "dct", 3),
             (oracle.REDFT11, "dct", 4), (oracle.RODFT00, "dst", 1), (oracle.RODFT10, "dst", 2),
             (oracle.RODFT01, "dst", 3), (oracle.RODFT11, "dst", 4)]
    for kind, fam, t in kinds:
        ref = getattr(scipy_fft, fam)(x, type=t)
        assert rel_l2(oracle.r2r(kind, x), ref) < 5e-15, (fam, t)


def test_c2r_ignores_imaginary_dc_and_nyquist(oracle):
    n = 10
    X = seeded_field((n // 2 + 1,), seed=1, dtype=np.complex128)
    Y = X.copy()
    Y[0] = Y[0].real
    Y[-1] = Y[-1].real
    assert np.array_equal(oracle.dft_c2r(X, n), oracle.dft_c2r(Y, n))


def test_type_registry(oracle):
    """IDs 0..43 in the order of p3dfft::setup (build/init.C:121-731); the DCT4 IDs run REDFT00
    because they are registered with the DCT1 planners (init.C:640-676)."""
    info = [oracle.type_info(i) for i in range(44)]
    assert [t["kind"] for t in info[:12]] == [0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4]
    assert [t["prec"] for t in info[:4]] == [4, 8, 4, 8]
    fam = [oracle.REDFT00, oracle.RODFT00, oracle.REDFT10, oracle.RODFT10, oracle.REDFT01, oracle.RODFT01,
           oracle.REDFT00, oracle.RODFT11]
    for f in range(8):
        for v in range(4):
            t = info[12 + 4 * f + v]
            assert t["kind"] == 5 and t["r2r"] == fam[f]
            assert t["dt1"] == t["dt2"] == (2 if v >= 2 else 1)
            assert t["prec"] == (8 if v & 1 else 4)
    with pytest.raises(ValueError):
        oracle.type_info(44)


def test_swap0_table(oracle):
    """swap0 (build/templ.C:816-858): L already stride-1 -> unchanged; rank 1 -> swap with the
    stride-1 dim; rank 2 -> rotate every rank by one."""
    for mo in itertools.permutations(range(3)):
        for L in range(3):
            new = oracle.swap0(mo, L)
            assert new[L] == 0
            if mo[L] == 0:
                assert new == mo
            elif mo[L] == 1:
                assert sorted(new) == [0, 1, 2] and new[mo.index(0)] == 1
            else:
                assert new == tuple((m + 1) % 3 for m in mo)


def _sine_field(n):
    t = np.arange(n) * 2 * np.pi / n
    s = np.sin(t)
    return np.ascontiguousarray(s[None, None, :] * s[None, :, None] * s[:, None, None]), t


def test_sample_test3D_r2c_known_answer(oracle):
    """sample/C++/test3D_r2c.C: +-0.125i at (+-1,+-1,+-1) after 1/N^3, max-abs within 1e-14*N/4;
    the round trip within 1e-14*Nglob/4."""
    n = 32
    x, _ = _sine_field(n)
    f = oracle.OraclePlan([5, 9, 9], (n, n, n), (0, 1, 2), (n // 2 + 1, n, n), (1, 2, 0), -1, 0)
    b = oracle.OraclePlan([7, 11, 11], (n // 2 + 1, n, n), (1, 2, 0), (n, n, n), (0, 1, 2), 0, -1)
    y = f.exec(x) / n ** 3
    ref = np.zeros_like(y)
    for ky, kz in itertools.product([1, n - 1], [1, n - 1]):
        ref[ky, 1, kz] = 0.125j * (1 if ky == 1 else -1) * (1 if kz == 1 else -1)
    assert np.max(np.abs(y - ref)) < 1e-14 * n * 0.25
    assert np.max(np.abs(b.exec(y) - x)) < 1e-14 * n ** 3 * 0.25


def test_sample_test_deriv_known_answer(oracle):
    """sample/C++/test_deriv.C: exec_deriv(idir) then backward gives cos in dimension idir."""
    n = 16
    x, t = _sine_field(n)
    f = oracle.OraclePlan([5, 9, 9], (n, n, n), (0, 1, 2), (n // 2 + 1, n, n), (1, 2, 0), -1, 0)
    b = oracle.OraclePlan([7, 11, 11], (n // 2 + 1, n, n), (1, 2, 0), (n, n, n), (0, 1, 2), 0, -1)
    s, c = np.sin(t), np.cos(t)
    for idir in range(3):
        z = b.exec(f.exec(x, idir=idir) / n ** 3)
        fac = [s, s, s]
        fac[idir] = c
        ref = fac[0][None, None, :] * fac[1][None, :, None] * fac[2][:, None, None]
        assert np.max(np.abs(z - ref)) < 1e-14 * n ** 3 * 0.25


@pytest.mark.parametrize("n", [9, 33, 129])
@pytest.mark.parametrize("dim", [0, 1, 2])
def test_sample_test1D_cos_sin_known_answers(oracle, n, dim):
    """sample/C++/test1D_cos.C: DCT-I of cos(pi x/(N-1)) times 0.5/(N-1) is 0.5 at index 1;
    test1D_sin.C: DST-I of sin(pi (x+1)/(N+1)) times 0.5/(N+1) is 0.5 at index 0."""
    gd = [4, 4, 4]
    gd[dim] = n
    mo = (0, 1, 2)
    shape = oracle.storage_shape(gd, mo)
    xs = np.arange(n)
    bshape = [1, 1, 1]
    bshape[2 - dim] = n
    for tid, wave, norm, peak in ((13, np.cos(xs * np.pi / (n - 1)), 0.5 / (n - 1), 1),
                                  (17, np.sin((xs + 1) * np.pi / (n + 1)), 0.5 / (n + 1), 0)):
        x = np.ascontiguousarray(np.broadcast_to(wave.reshape(bshape), shape))
        y = oracle.exec_stage(tid, dim, gd, mo, gd, mo, x) * norm
        ref = np.zeros(n)
        ref[peak] = 0.5
        ref = np.broadcast_to(ref.reshape(bshape), shape)
        assert np.max(np.abs(y - ref)) < 1e-14 * n * 0.25


def test_golden_fixtures(oracle):
    """The oracle reproduces the committed golden vectors (made by tests/golden/make_golden.py
    and cross-checked there against scipy.fft)."""
    g = np.load(GOLDEN)
    for name in sorted({k.rsplit("__", 1)[0] for k in g.files}):
        meta = g[name + "__meta"]
        x = g[name + "__in"]
        y = g[name + "__out"]
        types = [int(v) for v in meta[:3]]
        gd1, mo1, dcs1 = tuple(meta[3:6]), tuple(meta[6:9]), int(meta[9])
        gd2, mo2, dcs2 = tuple(meta[10:13]), tuple(meta[13:16]), int(meta[16])
        idir = int(meta[17])
        got = oracle.OraclePlan(types, gd1, mo1, gd2, mo2, dcs1, dcs2).exec(x, idir=idir)
        assert rel_l2(got, y) < 1e-14, name


@pytest.mark.parametrize("gd", [(16, 12, 10), (24, 18, 7), (30, 5, 9), (2, 3, 4), (10, 9, 33), (50, 1, 6)])
def test_batched_line_engine_equals_line_by_line(oracle, gd):
    """The oracle's batched line engine (blocks of 16 lines, Stockham radix 4 / 2 / 3 and direct
    odd radices, half-length R2C / C2R) against its line-by-line engine: R2C / C2C forward with
    each derivative dim, C2C backward, and the C2R round trip, over three memory-order pairs."""
    worst = 0.0
    for mo1, mo2 in [((0, 1, 2), (1, 2, 0)), ((2, 0, 1), (0, 1, 2)), ((1, 0, 2), (2, 1, 0))]:
        for fw, real in [((5, 9, 9), True), ((9, 9, 9), False), ((11, 11, 11), False)]:
            gd2 = (gd[0] // 2 + 1, gd[1], gd[2]) if real else gd
            p = oracle.OraclePlan(fw, gd, mo1, gd2, mo2, -1, 0 if real else -1)
            x = seeded_field(oracle.storage_shape(gd, mo1), seed=sum(gd) + mo1[0],
                             dtype=np.float64 if real else np.complex128)
            try:
                for idir in (-1, 0, 1, 2):
                    oracle.set_batched(False)
                    a = p.exec(x, idir=idir)
                    oracle.set_batched(True)
                    worst = max(worst, rel_l2(p.exec(x, idir=idir), a))
                if real:
                    pb = oracle.OraclePlan((7, 11, 11), gd2, mo2, gd, mo1, 0, -1)
                    s = p.exec(x)
                    oracle.set_batched(False)
                    a = pb.exec(s)
                    oracle.set_batched(True)
                    b = pb.exec(s)
                    worst = max(worst, rel_l2(b, a))
                    assert rel_l2(b / np.prod(gd), x) < 1e-14
            finally:
                oracle.set_batched(True)
    assert worst < 1e-14, worst
