"""CPU: the oracle against the reference's own outputs stored in tests/golden/ref_golden.npz.

The fixtures were written by tests/golden/make_ref_golden.py from the reference built here
(oracle/_ref); this test needs only the fixture file, so it runs on any machine.  It shows that the
oracle, which the GPU parity tests also use, reproduces the reference on every stored case: 3D
transforms over all memory-order pairs, fused derivatives, every 1D type (the D1 input-order
reinterpretation by its model: the oracle run on the input read in order swap0(mo1, dim)),
compute_deriv along the reference's storage axis (D7), and the 64^3, 384x256x257 and 512^3
(forward with fused d/dz) configurations by fingerprint.
"""
import json
import os

import numpy as np
import pytest

import refpin as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz")


def rel(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    return z, json.loads(str(z["meta"]))


def test_small_cases(oracle, golden):
    z, metas = golden
    kinds = {}
    for i, m in enumerate(metas):
        if m["kind"] == "3d":
            types = tuple(m["types"])
            prec = R.prec_of(types[0])
            x = R.det_field(R.storage_shape(m["g1"], m["mo1"]), m["seed"], R.input_is_complex(types), prec)
            y = oracle.OraclePlan(types, m["g1"], m["mo1"], m["g2"], m["mo2"], m["dcs1"], m["dcs2"]).exec(
                x, idir=m["idir"])
            tol = 1e-6 if prec == 4 else 1e-15
        elif m["kind"] == "1d":
            tid, dim = m["type"], m["dim"]
            prec = R.prec_of(tid)
            x = R.det_field(R.storage_shape(m["g1"], m["mo1"]), m["seed"], R.dt_of(tid)[0] == 2, prec)
            mo1 = R.swap0(m["mo1"], dim) if m["d1"] else tuple(m["mo1"])
            y = oracle.exec_stage(tid, dim, m["g1"], mo1, m["g2"], m["mo2"], x.reshape(R.storage_shape(m["g1"], mo1)))
            tol = 1e-6 if prec == 4 else 1e-15
        elif m["kind"] == "cderiv":
            x = R.det_field(R.storage_shape(m["g"], m["mo"]), m["seed"], True)
            y = oracle.compute_deriv(x, m["g"], m["mo"], m["dcs"], m["idir"], ref_axis=True)
            tol = 0.0
        else:
            continue
        ref = z[f"c{i}"]
        assert y.shape == ref.shape, m
        assert rel(y, ref) <= tol, (m, rel(y, ref))
        kinds[m["kind"]] = kinds.get(m["kind"], 0) + 1
    assert kinds.get("3d", 0) > 250 and kinds.get("1d", 0) > 80 and kinds.get("cderiv", 0) == 36, kinds


@pytest.mark.parametrize("name", ["config1", "config3", "config2"])
def test_full_size_configuration(oracle, golden, name):
    z, metas = golden
    cases = [(i, m) for i, m in enumerate(metas) if m["kind"] == "config" and m["name"] == name]
    if not cases:
        pytest.skip(f"{name} not in the fixture file")
    i, m = cases[0]
    types = tuple(m["types"])
    x = R.det_field(R.storage_shape(m["g1"], m["mo1"]), m["seed"], False)
    y = oracle.OraclePlan(types, m["g1"], m["mo1"], m["g2"], m["mo2"], m["dcs1"], m["dcs2"]).exec(x, idir=m["idir"])
    del x
    ref = {k: z[f"c{i}_{k}"] for k in ("idx", "val", "proj", "norm")}
    # (the oracle's batched line engine rounds differently from the reference's per-line FFTs:
    # 1.05e-15 on the 512^3 configuration, within 1e-15 line by line)
    assert R.fingerprint_error(R.fingerprint(y), ref) <= 4e-15
