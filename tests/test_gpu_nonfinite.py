"""GPU: lines of a stage stay independent, as in the reference's FFTW path (each 1D transform
is its own FFTW call).  The float-float kernels scale a tile of lines by a power of two taken
from its largest exponent; a tile whose lines differ widely in magnitude, or that holds an
infinity or NaN, scales each line by its own power of two taken from its finite values.  So an
infinity or NaN reaches every output of its own line and no other, and a line far smaller than
its tile neighbours keeps its relative accuracy."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

N = 512


def _field(dtype, seed=9):
    rng = np.random.default_rng(seed)
    shape = (3, 8, N)  # storage order (z, y, x) for memory order (0,1,2): 24 lines along x
    x = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    return x.astype(dtype)


@pytest.mark.parametrize("form", ["D_ff", "D_native", "S"])
def test_nonfinite_values_stay_in_their_line(gpu, oracle, form):
    p3d = gpu
    p3d.set_fp64_arith(0 if form == "D_native" else 1)
    tid = p3d.CFFT_FORWARD_S if form == "S" else p3d.CFFT_FORWARD_D
    cdt = np.complex64 if form == "S" else np.complex128
    g = (N, 8, 3)
    x = _field(cdt)
    bad = {(0, 5): (7, np.nan), (1, 2): (100, np.inf), (2, 6): (0, -np.inf)}
    xb = x.copy()
    for (z, y), (i, v) in bad.items():
        xb[z, y, i] = v + 0j
    tp = p3d.TransPlan(tid, g, (0, 1, 2), g, (0, 1, 2), 0)
    out = np.empty_like(xb)
    tp.exec(np.ascontiguousarray(xb), out)
    ref = oracle.exec_stage(p3d.CFFT_FORWARD_D, 0, g, (0, 1, 2), g, (0, 1, 2), x.astype(np.complex128))
    tol = 5e-6 if form == "S" else 1e-12
    for z in range(3):
        for y in range(8):
            line = out[z, y]
            if (z, y) in bad:
                assert not np.isfinite(line).any(), (z, y)
            else:
                assert np.isfinite(line).all(), (z, y)
                assert rel_l2(line, ref[z, y]) < tol, (z, y, rel_l2(line, ref[z, y]))


@pytest.mark.parametrize("form", ["D_ff", "D_native"])
def test_lines_of_a_tile_keep_their_own_precision(gpu, oracle, form):
    """Lines 1e300 apart in magnitude inside one tile: each line's result is accurate relative to
    its own norm (the float-float kernels scale every line by its own power of two)."""
    p3d = gpu
    p3d.set_fp64_arith(0 if form == "D_native" else 1)
    g = (N, 8, 3)
    x = _field(np.complex128, seed=10)
    mags = np.array([1e150, 1e-150, 1.0, 1e-300 * 1e10])  # repeated over the lines
    scale = np.resize(mags, 24).reshape(3, 8, 1)
    x = x * scale
    for tid, kind in ((p3d.CFFT_FORWARD_D, "C2C"), (p3d.CFFT_BACKWARD_D, "C2C")):
        tp = p3d.TransPlan(tid, g, (0, 1, 2), g, (0, 1, 2), 0)
        out = np.empty_like(x)
        tp.exec(np.ascontiguousarray(x), out)
        ref = oracle.exec_stage(tid, 0, g, (0, 1, 2), g, (0, 1, 2), x)
        for z in range(3):
            for y in range(8):
                assert rel_l2(out[z, y], ref[z, y]) < 1e-12, (kind, z, y, scale[z, y, 0])
