"""GPU: the autotuner's kernel choices.  Every (engine, tile-dim) choice a stage admits must give
the oracle's result (1e-12 relative L2 in float-float FP64, 2e-6 in FP32); tuning a plan records a
measured choice per stage, the result matches the heuristic plan, and the tuning cache round-trips
through its file."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

ENGINES = (1, 2, 3)  # specialised, register engine, generic


def _case(n, kind, orient):
    tid, lin, lout = {"c2c": (9, n, n), "r2c": (5, 2 * n, n + 1), "c2r": (7, n + 1, 2 * n)}[kind]
    if orient == "L":
        dim, mo1, mo2, g1, g2 = 0, (0, 1, 2), (0, 1, 2), (lin, 7, 5), (lout, 7, 5)
    else:
        dim, mo1, mo2, g1, g2 = 1, (0, 1, 2), (1, 0, 2), (11, lin, 6), (11, lout, 6)
    return tid, dim, mo1, mo2, g1, g2


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("kind", ["c2c", "r2c", "c2r"])
def test_every_engine_choice_matches_oracle(gpu, oracle, kind, prec):
    p3d = gpu
    p3d.set_fp64_arith(1)
    ran = 0
    for n in (64, 60, 56, 256):
        for orient in ("L", "t"):
            tid, dim, mo1, mo2, g1, g2 = _case(n, kind, orient)
            rng = np.random.default_rng(n)
            shape = p3d.storage_shape(g1, mo1)
            x = rng.uniform(-1, 1, shape) if tid == 5 else rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
            ref = oracle.exec_stage(tid, dim, g1, mo1, g2, mo2, x)
            t = tid if prec == 8 else tid - 1
            src = x if prec == 8 else x.astype(np.float32 if tid == 5 else np.complex64)
            odt = ref.dtype if prec == 8 else (np.float32 if ref.dtype == np.float64 else np.complex64)
            for eng in ENGINES:
                for talt in (0, 1):
                    tp = p3d.TransPlan(t, g1, mo1, g2, mo2, dim)
                    tp.set_engine(0, eng, talt)
                    out = np.empty(ref.shape, odt)
                    try:
                        tp.exec(np.ascontiguousarray(src), out)
                    except p3d.P3DFFTError as e:
                        assert "UNSUPPORTED" in str(e), (n, kind, orient, eng, talt, str(e))
                        continue
                    ran += 1
                    tol = 1e-12 if prec == 8 else 2e-6
                    assert rel_l2(out, ref) < tol, (n, kind, orient, eng, talt)
    assert ran >= 16


def test_autotune_plan_and_cache_file(gpu, oracle, tmp_path):
    p3d = gpu
    p3d.set_fp64_arith(1)
    p3d.tune_cache_clear()
    gd, gd2 = (64, 48, 40), (33, 48, 40)
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    x = np.random.default_rng(1).uniform(-1, 1, (40, 48, 64))
    y0 = f.exec(x)
    tun = f.autotune()
    assert len(tun) == 3 and all(e in ENGINES and ms > 0 for e, _, ms in tun), tun
    y1 = f.exec(x)
    assert rel_l2(y1, y0) < 1e-13
    ref = oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x)
    assert rel_l2(y1, ref) < 1e-12
    path = str(tmp_path / "tune.txt")
    p3d.tune_cache_save(path)
    p3d.tune_cache_clear()
    assert p3d.tune_cache_load(path) >= 3
    g = p3d.Transform3D(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    tun2 = g.autotune()  # served from the loaded cache: same choices and recorded times
    assert [(e, t) for e, t, _ in tun2] == [(e, t) for e, t, _ in tun]
    assert np.allclose([m for _, _, m in tun2], [m for _, _, m in tun], rtol=1e-6)


def test_autotune_at_first_exec(gpu):
    p3d = gpu
    p3d.set_fp64_arith(1)
    p3d.set_autotune(True)
    try:
        gd, gd2 = (40, 30, 24), (21, 30, 24)
        f = p3d.Transform3D([p3d.R2CFFT_S, p3d.CFFT_FORWARD_S, p3d.CFFT_FORWARD_S], gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
        assert all(e == 0 for e, _, _ in f.tuning())
        f.exec(np.random.default_rng(2).uniform(-1, 1, (24, 30, 40)).astype(np.float32))
        assert all(e in ENGINES for e, _, _ in f.tuning())
    finally:
        p3d.set_autotune(False)
