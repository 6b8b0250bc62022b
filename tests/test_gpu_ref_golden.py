"""GPU: the CUDA path against outputs of the reference itself (tests/golden/ref_golden.npz).

The fixtures were written by tests/golden/make_ref_golden.py from the reference's own
build/*.C compiled unchanged (oracle/_ref), so these tests pin the GPU path to the reference's
planner, memory-order reorders, derivative and 1D layouts, not to a restatement of them:

- 3D exec of 7 type sets over all 36 memory-order pairs, and exec_deriv where the reference is
  sound (full outputs, 6x5x4 grid);
- every 1D type ID, including plans whose input order the reference reinterprets (D1) and the
  reference's compute_deriv axis choice (D7), both reproduced in the library's default
  reference-compatible mode;
- the 64^3 and 384x256x257 configurations and the 512^3 forward transform with the fused d/dz
  derivative, through a size-independent fingerprint (sample values, +-1 projections, norm).
Tolerance: 1e-12 relative L2 for FP64 (1e-6 for FP32 plans, whose reference values are FP64
arithmetic rounded per stage).  Inputs are regenerated from the stored seeds (refpin.det_field).
"""
import json
import os

import numpy as np
import pytest

import refpin as R

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz")


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    return z, json.loads(str(z["meta"]))


@pytest.fixture
def compat(gpu):
    gpu.set_reference_compat(True)
    yield gpu
    gpu.set_reference_compat(False)


def rel(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _cases(golden, pred):
    z, metas = golden
    return [(i, m) for i, m in enumerate(metas) if pred(m)]


SETS = ["r2c_c2c_c2c", "c2r_c2c_c2c", "c2c_forward", "r2c_c2c_dct1", "real_dct2_dst2_dct3", "r2c_c2c_empty",
        "r2c_single", "r2c_deriv"]


@pytest.mark.parametrize("name", SETS)
def test_3d_against_reference(compat, golden, name):
    p3d = compat
    z, _ = golden
    cases = _cases(golden, lambda m: m["kind"] == "3d" and m["set"] == name)
    assert len(cases) >= 30
    worst = 0.0
    for i, m in cases:
        types = tuple(m["types"])
        prec = R.prec_of(types[0])
        x = R.det_field(R.storage_shape(m["g1"], m["mo1"]), m["seed"], R.input_is_complex(types), prec)
        f = p3d.Transform3D(types, m["g1"], m["mo1"], m["g2"], m["mo2"], m["dcs1"], m["dcs2"])
        y = f.exec(x, idir=m["idir"])
        ref = z[f"c{i}"]
        assert y.shape == ref.shape, (m, y.shape, ref.shape)
        e = rel(y, ref)
        assert e <= (1e-6 if prec == 4 else 1e-12), (m, e)
        worst = max(worst, e)
    print(f"{name}: {len(cases)} cases, worst relative L2 {worst:.2e}")


def test_1d_every_type_against_reference(compat, golden):
    p3d = compat
    z, _ = golden
    cases = _cases(golden, lambda m: m["kind"] == "1d")
    assert len(cases) >= 80 and any(m["d1"] for _, m in cases)
    for i, m in cases:
        tid, prec = m["type"], R.prec_of(m["type"])
        dt1, dt2 = R.dt_of(tid)
        x = R.det_field(R.storage_shape(m["g1"], m["mo1"]), m["seed"], dt1 == 2, prec)
        y = np.empty(R.storage_shape(m["g2"], m["mo2"]),
                     (np.complex128 if prec == 8 else np.complex64) if dt2 == 2 else
                     (np.float64 if prec == 8 else np.float32))
        p3d.TransPlan(tid, m["g1"], m["mo1"], m["g2"], m["mo2"], m["dim"]).exec(x, y)
        e = rel(y, z[f"c{i}"])
        assert e <= (1e-6 if prec == 4 else 1e-12), (m, e)


def test_compute_deriv_against_reference(compat, golden):
    p3d = compat
    z, _ = golden
    cases = _cases(golden, lambda m: m["kind"] == "cderiv")
    assert len(cases) == 36
    for i, m in cases:
        x = R.det_field(R.storage_shape(m["g"], m["mo"]), m["seed"], True)
        y = np.empty_like(x)
        p3d.compute_deriv(x, y, m["g"], m["mo"], m["dcs"], m["idir"])
        assert rel(y, z[f"c{i}"]) <= 1e-15, m


def test_compute_deriv_corrected_axis_differs_only_for_3_cycles(gpu, golden):
    """With reference compatibility off the derivative follows logical dim idir: identical to the
    reference for identity / transposition orders, different for the 3-cycles."""
    p3d = gpu
    p3d.set_reference_compat(False)
    z, _ = golden
    for i, m in _cases(golden, lambda m: m["kind"] == "cderiv"):
        x = R.det_field(R.storage_shape(m["g"], m["mo"]), m["seed"], True)
        y = np.empty_like(x)
        p3d.compute_deriv(x, y, m["g"], m["mo"], m["dcs"], m["idir"])
        e = rel(y, z[f"c{i}"])
        if R.inv_mo(m["mo"]) == tuple(m["mo"]):
            assert e <= 1e-15, m
        else:
            assert e > 1e-2, m


@pytest.mark.parametrize("name", ["config1", "config3", "config2"])
def test_full_size_configuration_against_reference(compat, golden, name):
    p3d = compat
    z, metas = golden
    cases = _cases(golden, lambda m: m["kind"] == "config" and m["name"] == name)
    if not cases:
        pytest.skip(f"{name} not in the fixture file")
    i, m = cases[0]
    types = tuple(m["types"])
    x = R.det_field(R.storage_shape(m["g1"], m["mo1"]), m["seed"], False)
    f = p3d.Transform3D(types, m["g1"], m["mo1"], m["g2"], m["mo2"], m["dcs1"], m["dcs2"])
    y = f.exec(x, idir=m["idir"])
    del x
    ref = {k: z[f"c{i}_{k}"] for k in ("idx", "val", "proj", "norm")}
    e = R.fingerprint_error(R.fingerprint(y), ref)
    print(f"{name}: fingerprint error vs the reference {e:.2e}")
    assert e <= 1e-12, e
