"""GPU: FP32 split (compensated) twiddle products on the long lines.

FP32 stages whose FFT length is 512, 1024 or 2048 multiply by twiddles stored as FP32 pairs
(hi, lo) whose sum is the long-double value, as a * hi + a * lo; shorter lines keep FP32 twiddles
(most formed as products of two table entries).  Against the FP64 oracle, per line length and
kind: the FP32 error stays within 1e-6 relative L2 either way, and the split form is no worse
than the plain form on the long lines (it removes the twiddles' own roundings).  The errors are
printed per length.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu

LENGTHS = [64, 256, 512, 1024, 2048]


def _run(p3d, oracle, tid_s, tid_d, n, split, seed):
    p3d.set_fp32_split_twiddles(split)
    g = (n, 24, 8)
    kind = {p3d.CFFT_FORWARD_S: "c2c", p3d.R2CFFT_S: "r2c", p3d.C2RFFT_S: "c2r"}[tid_s]
    g1, g2 = list(g), list(g)
    if kind == "r2c":
        g2[0] = n // 2 + 1
    if kind == "c2r":
        g1[0] = n // 2 + 1
    cplx = kind != "r2c"
    x = seeded_field(p3d.storage_shape(g1, (0, 1, 2)), seed=seed, dtype=np.complex64 if cplx else np.float32)
    if kind == "c2r":  # a Hermitian-consistent spectrum: DC and Nyquist real
        x[..., 0] = x[..., 0].real
        x[..., -1] = x[..., -1].real
    y = np.empty(p3d.storage_shape(g2, (0, 1, 2)), np.float32 if kind == "c2r" else np.complex64)
    p3d.TransPlan(tid_s, tuple(g1), (0, 1, 2), tuple(g2), (0, 1, 2), 0).exec(np.ascontiguousarray(x), y)
    ref = oracle.exec_stage(tid_d, 0, tuple(g1), (0, 1, 2), tuple(g2), (0, 1, 2),
                            x.astype(np.complex128 if cplx else np.float64))
    return rel_l2(y, ref)


@pytest.mark.parametrize("kind", ["c2c", "r2c", "c2r"])
def test_split_twiddles_error_per_length(gpu, oracle, kind):
    p3d = gpu
    tids = {"c2c": (p3d.CFFT_FORWARD_S, p3d.CFFT_FORWARD_D), "r2c": (p3d.R2CFFT_S, p3d.R2CFFT_D),
            "c2r": (p3d.C2RFFT_S, p3d.C2RFFT_D)}[kind]
    try:
        for n in LENGTHS:
            e_split = _run(p3d, oracle, tids[0], tids[1], n, True, 100 + n)
            e_plain = _run(p3d, oracle, tids[0], tids[1], n, False, 100 + n)
            nfft = n // 2 if kind in ("r2c", "c2r") else n
            print(f"{kind} n={n}: FP32 rel L2 vs FP64 oracle, split {e_split:.2e}, plain {e_plain:.2e}")
            assert e_split < 1e-6 and e_plain < 1e-6, (n, e_split, e_plain)
            if nfft >= 512:
                assert e_split <= 1.02 * e_plain, (n, e_split, e_plain)
            else:
                assert e_split == e_plain, n  # short lines: the same kernel either way
    finally:
        p3d.set_fp32_split_twiddles(True)
