"""GPU: the edges of the supported sizes.

- Long lines against the CPU oracle (1e-12 relative L2 in FP64, 5e-6 in FP32): the longest a
  stage takes (6144 points FP64, 12288 FP32), 4096 and 8192 points (past the register engine),
  primes on the Bluestein engine at its largest convolution (2039 FP64, 4093 FP32) and primes
  past it on the generic radix engine (4093 and 6143 FP64, one DFT of the whole line); one point
  past the limit rejected with P3DFFT_ERR_TOO_LARGE, leaving the library usable.
- Degenerate 3D grids (dims of 1 and 2 in every position, R2C of length 1 and 2) against the
  oracle.
(Plans the reference cannot form either, a zero dim or a C2R to a real length of 1, are rejected
at plan time: `tests/test_host_runtime.py`.)
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu


def _line(p3d, oracle, tid_d, prec, n, lines=(3, 2)):
    g = (n, lines[0], lines[1])
    x = seeded_field(p3d.storage_shape(g, (0, 1, 2)), seed=n, dtype=np.complex128)
    ref = oracle.exec_stage(tid_d, 0, g, (0, 1, 2), g, (0, 1, 2), x)
    tid = tid_d if prec == 8 else tid_d - 1
    tp = p3d.TransPlan(tid, g, (0, 1, 2), g, (0, 1, 2), 0)
    src = x if prec == 8 else x.astype(np.complex64)
    out = np.empty(ref.shape, np.complex128 if prec == 8 else np.complex64)
    tp.exec(np.ascontiguousarray(src), out)
    return rel_l2(out, ref)


@pytest.mark.parametrize("prec,n", [(8, 6144), (8, 4096), (8, 2039), (8, 4093), (8, 6143), (4, 12288), (4, 8192),
                                    (4, 4093)])
def test_longest_lines_against_oracle(gpu, oracle, prec, n):
    p3d = gpu
    p3d.set_fp64_arith(1)
    err = _line(p3d, oracle, p3d.CFFT_FORWARD_D, prec, n)
    assert err < (1e-12 if prec == 8 else 5e-6), (prec, n, err)


@pytest.mark.parametrize("prec,n", [(8, 6145), (4, 12289)])
def test_one_point_past_the_limit_is_rejected(gpu, oracle, prec, n):
    p3d = gpu
    with pytest.raises(p3d.P3DFFTError, match="TOO_LARGE"):
        _line(p3d, oracle, p3d.CFFT_FORWARD_D, prec, n, lines=(1, 1))
    # the library stays usable
    assert _line(p3d, oracle, p3d.CFFT_FORWARD_D, prec, 64) < (1e-12 if prec == 8 else 5e-6)


# R2C / C2R need an even real length: the reference sizes a C2R output 2(M-1) from M complex
# points (templ.C:274-277), so a real length of 1 has no C2R stage (tested below as an error)
GRIDS = [(2, 1, 1), (2, 2, 2), (2, 7, 5), (6, 1, 5), (6, 5, 1), (2, 16, 16)]
CGRIDS = [(1, 1, 1), (1, 2, 1), (1, 1, 2), (1, 7, 5), (5, 1, 1), (1, 16, 16)]


@pytest.mark.parametrize("gd", GRIDS, ids=[f"{g[0]}x{g[1]}x{g[2]}" for g in GRIDS])
@pytest.mark.parametrize("mo2", [(0, 1, 2), (1, 2, 0)])
def test_degenerate_grids_round_trip(gpu, oracle, gd, mo2):
    """R2C/C2C/C2C forward with d/dz and C2R/C2C/C2C back on grids with dims of 1 and 2."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, mo2, -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, mo2, gd, (0, 1, 2), 0, -1)
    x = seeded_field(f.in_shape(), seed=sum(gd), dtype=np.float64)
    spec = f.exec(x, idir=2)
    ref = oracle.OraclePlan([5, 9, 9], gd, (0, 1, 2), gd2, mo2, -1, 0).exec(x, idir=2)
    assert rel_l2(spec, ref) < 1e-12 or np.linalg.norm(ref) == 0
    y = b.exec(spec)
    yref = oracle.OraclePlan([7, 11, 11], gd2, mo2, gd, (0, 1, 2), 0, -1).exec(ref)
    assert rel_l2(y, yref) < 1e-12 or np.linalg.norm(yref) == 0


@pytest.mark.parametrize("gd", CGRIDS, ids=[f"{g[0]}x{g[1]}x{g[2]}" for g in CGRIDS])
@pytest.mark.parametrize("prec", [8, 4])
def test_degenerate_grids_c2c(gpu, oracle, gd, prec):
    """C2C in all three dims with d/dy on grids with dims of 1, FP64 and FP32."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    types = [p3d.CFFT_FORWARD_D] * 3 if prec == 8 else [p3d.CFFT_FORWARD_S] * 3
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd, (2, 1, 0), -1, -1)
    x = seeded_field(f.in_shape(), seed=7 + sum(gd), dtype=np.complex128)
    y = f.exec(x if prec == 8 else x.astype(np.complex64), idir=1)
    ref = oracle.OraclePlan([9, 9, 9], gd, (0, 1, 2), gd, (2, 1, 0), -1, -1).exec(x, idir=1)
    assert rel_l2(y, ref) < (1e-12 if prec == 8 else 1e-6) or np.linalg.norm(ref) == 0
