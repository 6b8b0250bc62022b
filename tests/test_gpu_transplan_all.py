"""GPU: the 1D transplan interface for every one of the 44 transform type IDs (EMPTY, R2C, C2R,
C2C both directions, DCT/DST I-IV on real and complex data, single and double precision) over
all 36 (input, output) memory-order pairs, the transform dim cycling through 0, 1, 2.  Each case
is compared with the CPU oracle's stage (1e-12 relative L2 for FP64 in float-float, 5e-6 for
FP32).  Covers the reference's transplan<T1,T2> (build/templ.C:900-1075, exec.C:522-1326)."""
import itertools

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

PERMS = list(itertools.permutations(range(3)))
TYPE_NAMES = [
    "EMPTY_TYPE_SINGLE", "EMPTY_TYPE_DOUBLE", "EMPTY_TYPE_SINGLE_COMPLEX", "EMPTY_TYPE_DOUBLE_COMPLEX",
    "R2CFFT_S", "R2CFFT_D", "C2RFFT_S", "C2RFFT_D", "CFFT_FORWARD_S", "CFFT_FORWARD_D", "CFFT_BACKWARD_S",
    "CFFT_BACKWARD_D"] + [f"{k}{n}_{d}_{p}" for k in ("DCT", "DST") for n in (1, 2, 3, 4) for d in ("REAL", "COMPLEX")
                          for p in ("S", "D")]


def _d_id(oracle, p3d, name):
    """The FP64 type ID of the same transform (the oracle computes in double)."""
    return p3d.TYPE_IDS[name[:-1] + "D"] if name.endswith("_S") else p3d.TYPE_IDS[name]


@pytest.mark.parametrize("name", TYPE_NAMES)
def test_transplan_every_type_every_order(gpu, oracle, name):
    p3d = gpu
    p3d.set_fp64_arith(1)
    tid = p3d.TYPE_IDS[name]
    tid_d = _d_id(oracle, p3d, name)
    ti = oracle.type_info(tid)
    prec = ti["prec"]
    n = 12
    worst = 0.0
    for k, (mo1, mo2) in enumerate(itertools.product(PERMS, PERMS)):
        dim = k % 3
        g1, g2 = [5, 7, 6], [5, 7, 6]
        g1[dim] = g2[dim] = n
        if ti["dt1"] == 1 and ti["dt2"] == 2:  # R2C
            g2[dim] = n // 2 + 1
        elif ti["dt1"] == 2 and ti["dt2"] == 1:  # C2R
            g1[dim] = n // 2 + 1
        rng = np.random.default_rng(k)
        shape = p3d.storage_shape(g1, mo1)
        x = rng.uniform(-1, 1, shape)
        if ti["dt1"] == 2:
            x = x + 1j * rng.uniform(-1, 1, shape)
        ref = oracle.exec_stage(tid_d, dim, tuple(g1), mo1, tuple(g2), mo2, x)
        if prec == 4:
            src = x.astype(np.complex64 if ti["dt1"] == 2 else np.float32)
            out = np.empty(ref.shape, np.complex64 if ti["dt2"] == 2 else np.float32)
        else:
            src, out = x, np.empty_like(ref)
        tp = p3d.TransPlan(tid, tuple(g1), mo1, tuple(g2), mo2, dim)
        tp.exec(np.ascontiguousarray(src), out)
        e = rel_l2(out, ref)
        worst = max(worst, e)
        assert e < (1e-12 if prec == 8 else 5e-6), (name, mo1, mo2, dim, e)
    print(f"{name}: worst rel L2 {worst:.2e} over 36 order pairs")
