"""GPU: the specialised stage kernels at every FFT length they are built for (2^a 3^b 5^c from 16
to 512, plus 1024 and 2048), for C2C forward/backward, R2C and C2R, in the three arithmetics,
with the line along the stride-1 dim (L-major tile) and along a strided dim with a memory-order
change (t-major tile).  Each case is one 1D transplan stage compared with the CPU oracle's stage.

Tolerances (relative L2): 1e-12 for FP64 (float-float and native), 2e-6 for FP32."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

LENGTHS = [16, 18, 20, 24, 25, 27, 30, 32, 36, 40, 45, 48, 50, 54, 60, 64, 72, 75, 80, 81, 90, 96, 100, 108,
           120, 125, 128, 135, 144, 150, 160, 162, 180, 192, 200, 216, 225, 240, 243, 250, 256, 270, 288, 300,
           320, 324, 360, 375, 384, 400, 405, 432, 450, 480, 486, 500, 512, 1024, 2048]

# (name, D type id, logical length in, logical length out) for an FFT length n
KINDS = {
    "c2c_fwd": (9, lambda n: (n, n)),
    "c2c_bwd": (11, lambda n: (n, n)),
    "r2c": (5, lambda n: (2 * n, n + 1)),
    "c2r": (7, lambda n: (n + 1, 2 * n)),
}
ORIENT = {  # dim, mo1, mo2, other dims
    "Lmajor": (0, (0, 1, 2), (0, 1, 2), (6, 5)),
    "tmajor": (1, (0, 1, 2), (1, 0, 2), (37, 3)),
}


def _grids(dim, lin, lout, others):
    g1, g2 = [0, 0, 0], [0, 0, 0]
    o = iter(others)
    for d in range(3):
        if d == dim:
            g1[d], g2[d] = lin, lout
        else:
            g1[d] = g2[d] = next(o)
    return tuple(g1), tuple(g2)


def _input(p3d, tid_d, g1, mo1, seed):
    rng = np.random.default_rng(seed)
    shape = p3d.storage_shape(g1, mo1)
    if tid_d == 5:
        return rng.uniform(-1, 1, shape)
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


@pytest.mark.parametrize("orient", list(ORIENT))
@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("form", ["fp64_float_float", "fp64_native", "fp32"])
def test_fast_lengths_against_oracle(gpu, oracle, form, kind, orient):
    p3d = gpu
    p3d.set_fp64_arith(0 if form == "fp64_native" else 1)
    tid_d, lens = KINDS[kind]
    dim, mo1, mo2, others = ORIENT[orient]
    prec = 4 if form == "fp32" else 8
    tol = 2e-6 if prec == 4 else 1e-12
    worst = (0.0, None)
    for n in LENGTHS:
        if orient == "tmajor" and n > 512:
            others_n = (9, 2)  # keep the strided case small at the longest lengths
        else:
            others_n = others
        lin, lout = lens(n)
        g1, g2 = _grids(dim, lin, lout, others_n)
        x = _input(p3d, tid_d, g1, mo1, seed=n)
        ref = oracle.exec_stage(tid_d, dim, g1, mo1, g2, mo2, x)
        tid = tid_d if prec == 8 else tid_d - 1
        tp = p3d.TransPlan(tid, g1, mo1, g2, mo2, dim)
        if prec == 4:
            src = x.astype(np.complex64 if np.iscomplexobj(x) else np.float32)
            out = np.empty(ref.shape, np.complex64 if np.iscomplexobj(ref) else np.float32)
        else:
            src, out = x, np.empty_like(ref)
        tp.exec(np.ascontiguousarray(src), out)
        e = rel_l2(out, ref)
        if e > worst[0]:
            worst = (e, n)
        assert e < tol, (form, kind, orient, n, e)
    print(f"{form} {kind} {orient}: worst rel L2 {worst[0]:.2e} at N={worst[1]}")
