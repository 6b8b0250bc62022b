"""GPU: the DCT / DST kinds on the specialised kernels.

DCT-I / DST-I (FFTW REDFT00 / RODFT00, and the DCT4 IDs the reference registers with the DCT-I
planners, build/init.C:640-676) transform the line's even / odd extension with one FFT of length
2(n-1) / 2(n+1); real lines go two at a time as the real and imaginary parts of one complex line,
so line counts are chosen odd as well as even (the last line of an odd count is paired with
itself).  DCT / DST II-IV transform the pre-twiddled, zero-padded line with one FFT of length 2n.
Each case runs with the specialised engine forced and with the generic engine, and both are
compared with the CPU oracle's stage: 1e-12 relative L2 for FP64 (float-float and native), 5e-6
for FP32."""
import itertools

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

ENG_FAST, ENG_GENERIC = 1, 3
# (family, line length n): FFT lengths 2(n-1) for DCT-I, 2(n+1) for DST-I, all specialised
CASES = [("DCT1", 9), ("DCT1", 13), ("DCT1", 17), ("DCT1", 26), ("DCT1", 129), ("DCT1", 257),
         ("DST1", 7), ("DST1", 11), ("DST1", 15), ("DST1", 49), ("DST1", 255), ("DCT4", 33)]
ORDERS = [((0, 1, 2), (0, 1, 2)), ((0, 1, 2), (1, 2, 0)), ((2, 1, 0), (0, 2, 1)), ((1, 0, 2), (2, 0, 1))]


def _run(p3d, oracle, name, n, dim, mo1, mo2, others, engine, seed):
    tid = p3d.TYPE_IDS[name]
    tid_d = p3d.TYPE_IDS[name[:-1] + "D"]
    ti = oracle.type_info(tid)
    g = list(others)
    g.insert(dim, n)
    g = tuple(g)
    rng = np.random.default_rng(seed)
    shape = p3d.storage_shape(g, mo1)
    x = rng.uniform(-1, 1, shape)
    if ti["dt1"] == 2:
        x = x + 1j * rng.uniform(-1, 1, shape)
    ref = oracle.exec_stage(tid_d, dim, g, mo1, g, mo2, x)
    if ti["prec"] == 4:
        src = x.astype(np.complex64 if ti["dt1"] == 2 else np.float32)
        out = np.empty(ref.shape, np.complex64 if ti["dt2"] == 2 else np.float32)
    else:
        src, out = x, np.empty_like(ref)
    tp = p3d.TransPlan(tid, g, mo1, g, mo2, dim)
    tp.set_engine(0, engine)
    tp.exec(np.ascontiguousarray(src), out)
    return rel_l2(out, ref), ti["prec"]


@pytest.mark.parametrize("family,n", CASES)
@pytest.mark.parametrize("data", ["REAL", "COMPLEX"])
@pytest.mark.parametrize("form", ["D_ff", "D_native", "S"])
def test_dct1_dst1_specialised_vs_oracle(gpu, oracle, family, n, data, form):
    p3d = gpu
    p3d.set_fp64_arith(0 if form == "D_native" else 1)
    name = f"{family}_{data}_{form[0]}"
    worst = {ENG_FAST: 0.0, ENG_GENERIC: 0.0}
    for k, (mo1, mo2) in enumerate(ORDERS):
        dim = k % 3
        others = (5, 7) if k % 2 == 0 else (6, 4)  # 35 lines (odd) or 24 lines (even)
        for eng in (ENG_FAST, ENG_GENERIC):
            e, prec = _run(p3d, oracle, name, n, dim, mo1, mo2, others, eng, seed=1000 * n + k)
            worst[eng] = max(worst[eng], e)
    tol = 1e-12 if prec == 8 else 5e-6
    assert worst[ENG_FAST] < tol, worst
    assert worst[ENG_GENERIC] < tol, worst


def test_dct1_single_line_and_single_pair(gpu, oracle):
    """One real line (paired with itself), two real lines (one pair), three (a pair and a half)."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    for lines, name in itertools.product((1, 2, 3), ("DCT1_REAL_D", "DST1_REAL_D")):
        n = 17 if name.startswith("DCT") else 15
        e, _ = _run(p3d, oracle, name, n, 0, (0, 1, 2), (0, 1, 2), (lines, 1), ENG_FAST, seed=lines)
        assert e < 1e-12, (name, lines, e)


def test_config3_dct_stage_on_specialised_kernel(gpu):
    """The 384x256x257 plan's z stage (DCT-I, complex, n = 257) runs on the specialised kernels:
    with that engine forced on every stage the plan executes and agrees with the generic engine
    on the DCT stage."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd, gd2 = (384, 256, 257), (193, 256, 257)
    types = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.DCT1_COMPLEX_D]
    x = np.random.default_rng(257).uniform(-1, 1, p3d.storage_shape(gd, (0, 1, 2)))
    out = {}
    for eng in (ENG_FAST, ENG_GENERIC):
        f = p3d.Transform3D(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
        st = f.stages(executed=True)
        for s in range(len(st)):
            f.set_engine(s, eng if st[s]["type"] == p3d.DCT1_COMPLEX_D else ENG_FAST)
        out[eng] = f.exec(x)
    assert rel_l2(out[ENG_FAST], out[ENG_GENERIC]) < 1e-13


# DCT / DST II-IV on the specialised kernels (one FFT of length 2n of the pre-twiddled,
# zero-padded line): n with 2n among the specialised lengths
CASES_G = [(f, n) for f in ("DCT2", "DCT3", "DST2", "DST3", "DST4") for n in (8, 12, 25, 50, 256)]


@pytest.mark.parametrize("family,n", CASES_G)
@pytest.mark.parametrize("data", ["REAL", "COMPLEX"])
@pytest.mark.parametrize("form", ["D_ff", "D_native", "S"])
def test_dct_dst_2_3_4_specialised_vs_oracle(gpu, oracle, family, n, data, form):
    p3d = gpu
    p3d.set_fp64_arith(0 if form == "D_native" else 1)
    name = f"{family}_{data}_{form[0]}"
    worst = {ENG_FAST: 0.0, ENG_GENERIC: 0.0}
    for k, (mo1, mo2) in enumerate(ORDERS):
        dim = k % 3
        others = (5, 7) if k % 2 == 0 else (6, 4)
        for eng in (ENG_FAST, ENG_GENERIC):
            e, prec = _run(p3d, oracle, name, n, dim, mo1, mo2, others, eng, seed=2000 * n + k)
            worst[eng] = max(worst[eng], e)
    tol = 1e-12 if prec == 8 else 5e-6
    assert worst[ENG_FAST] < tol, worst
    assert worst[ENG_GENERIC] < tol, worst
