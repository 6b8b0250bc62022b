"""GPU: float-float intermediate fields between specialised float-float stages.

With float-float FP64 arithmetic, consecutive stages that both run the specialised kernels pass
their intermediate field as packed float-float pairs at per-line power-of-two scales (scales in a
side array) instead of IEEE doubles.  These tests check, through the C ABI, that this changes
nothing a caller can see beyond rounding:

- R2C / C2C / C2C with each fused derivative and the C2R way back: against the oracle (1e-12
  relative L2) and against the same plans with IEEE intermediates (1e-13);
- slabs whose magnitudes differ by up to 10^490 inside one intermediate field: each slab of a
  C2C / EMPTY / C2C plan (x and z transformed, the y slabs never mixed) keeps 1e-12 accuracy
  relative to its own norm, with float-float and with IEEE intermediates;
- infinities and NaNs reach exactly the slabs they are in, as with IEEE intermediates.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu


@pytest.fixture
def ff(gpu):
    gpu.set_fp64_arith(1)
    gpu.set_ff_intermediates(True)
    yield gpu
    gpu.set_ff_intermediates(True)


def _plans(p3d, gd):
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    return f, b, gd2


@pytest.mark.parametrize("gd", [(512, 64, 32), (64, 96, 80), (256, 128, 64)])
def test_round_trip_against_oracle_and_ieee_intermediates(ff, oracle, gd):
    p3d = ff
    f, b, gd2 = _plans(p3d, gd)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=71)
    fwd = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
    bwd = [p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D]
    of = oracle.OraclePlan(fwd, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    ob = oracle.OraclePlan(bwd, gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    for idir in (-1, 0, 1, 2):
        p3d.set_ff_intermediates(True)
        y = f.exec(x, idir=idir)
        z = b.exec(y)
        p3d.set_ff_intermediates(False)
        y0 = f.exec(x, idir=idir)
        z0 = b.exec(y0)
        yo = of.exec(x, idir=idir)
        assert rel_l2(y, yo) < 1e-12, (gd, idir, rel_l2(y, yo))
        assert rel_l2(z, ob.exec(yo)) < 1e-12, (gd, idir)
        assert rel_l2(y, y0) < 1e-13 and rel_l2(z, z0) < 1e-13, (gd, idir)


MO_PAIRS = [((2, 0, 1), (0, 1, 2)), ((1, 0, 2), (2, 1, 0)), ((0, 2, 1), (1, 0, 2)), ((1, 2, 0), (2, 0, 1))]


@pytest.mark.parametrize("mo1,mo2", MO_PAIRS, ids=[f"{a}-{b}" for a, b in MO_PAIRS])
def test_memory_orders_against_oracle(ff, oracle, mo1, mo2):
    """Float-float links between stages whose intermediate layouts follow other memory orders (the
    scale arrays are ordered for the consuming stage): against the oracle and IEEE intermediates,
    with d/dy fused."""
    p3d = ff
    gd = (128, 256, 64)
    gd2 = (65, 256, 64)
    fwd = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
    bwd = [p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D]
    f = p3d.Transform3D(fwd, gd, mo1, gd2, mo2, -1, 0)
    b = p3d.Transform3D(bwd, gd2, mo2, gd, mo1, 0, -1)
    x = seeded_field(p3d.storage_shape(gd, mo1), seed=73)
    y = f.exec(x, idir=1)
    z = b.exec(y)
    p3d.set_ff_intermediates(False)
    y0 = f.exec(x, idir=1)
    z0 = b.exec(y0)
    p3d.set_ff_intermediates(True)
    yo = oracle.OraclePlan(fwd, gd, mo1, gd2, mo2, -1, 0).exec(x, idir=1)
    zo = oracle.OraclePlan(bwd, gd2, mo2, gd, mo1, 0, -1).exec(yo)
    assert rel_l2(y, yo) < 1e-12 and rel_l2(z, zo) < 1e-12
    assert rel_l2(y, y0) < 1e-13 and rel_l2(z, z0) < 1e-13


# x and z transformed, y EMPTY: the x -> z boundary is a float-float intermediate and the y index
# (storage axis 1) separates slabs that no stage mixes
G_SLAB = (256, 8, 64)


def _slab_types(p3d):
    return [p3d.CFFT_FORWARD_D, p3d.EMPTY_TYPE_DOUBLE_COMPLEX, p3d.CFFT_FORWARD_D]


def _slab_plan(p3d):
    f = p3d.Transform3D(_slab_types(p3d), G_SLAB, (0, 1, 2), G_SLAB, (0, 1, 2))
    st = [s["type"] for s in f.stages(executed=True)]
    assert any(st[i] != p3d.EMPTY_TYPE_DOUBLE_COMPLEX and st[i + 1] != p3d.EMPTY_TYPE_DOUBLE_COMPLEX
               for i in range(len(st) - 1)), "no two transform stages are adjacent"
    return f


def test_slabs_far_apart_in_magnitude_keep_their_precision(ff, oracle):
    p3d = ff
    x = seeded_field(p3d.storage_shape(G_SLAB, (0, 1, 2)), seed=73, dtype=np.complex128)
    mags = np.array([1e150, 1e-150, 1.0, 1e-290, 1e200, 3e-5, 1e-100, 7.0])
    x = np.ascontiguousarray(x * mags.reshape(1, 8, 1))
    f = _slab_plan(p3d)
    ref = oracle.OraclePlan(_slab_types(p3d), G_SLAB, (0, 1, 2), G_SLAB, (0, 1, 2)).exec(x)
    for ffon in (True, False):
        p3d.set_ff_intermediates(ffon)
        y = f.exec(x)
        for k, m in enumerate(mags):  # compared at unit scale (squares of 1e200 overflow)
            e = rel_l2(y[:, k] / m, ref[:, k] / m)
            assert e < 1e-12, (ffon, k, m, e)


def test_nonfinite_values_stay_in_their_slab(ff):
    p3d = ff
    x = seeded_field(p3d.storage_shape(G_SLAB, (0, 1, 2)), seed=79, dtype=np.complex128)
    x[7, 1, 5] = np.nan
    x[0, 4, 100] = np.inf
    x[63, 6, 0] = -np.inf + 0j
    x = np.ascontiguousarray(x)
    f = _slab_plan(p3d)
    p3d.set_ff_intermediates(True)
    y = f.exec(x)
    p3d.set_ff_intermediates(False)
    y0 = f.exec(x)
    for k in range(8):
        if k in (1, 4, 6):
            assert not np.isfinite(y[:, k]).any(), k
        else:
            assert np.isfinite(y[:, k]).all(), k
            assert rel_l2(y[:, k], y0[:, k]) < 1e-13, k
    assert np.array_equal(np.isfinite(y), np.isfinite(y0))
