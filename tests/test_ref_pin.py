"""CPU: the oracle pinned to the reference itself.

oracle/_ref/libp3dfft_ref.so is the reference's own build/{init,templ,exec,deriv,wrap}.C compiled
unchanged (oracle/build_ref.py) with FFTW's 1D arithmetic supplied by oracle/refshim/fftw_shim.c.
These tests drive it through the reference's C interface (oracle/pyref.py) and check:

- the reference's own sample programs, built unchanged against it, print "Results are correct"
  (the shims give the reference the FFTW and MPI behaviour its checks expect);
- 3D exec: for every memory-order pair and several type sets (R2C/C2R, C2C, R2C+C2C+DCT-I, real
  DCT/DST, an EMPTY dim, single precision), the oracle's output equals the reference's;
- 3D exec_deriv: equal outside the reference's defects D4 (crash, checked in a child process) and
  D5 (wrong derivative in one reorder_deriv branch), where the reference is shown to differ;
- every 1D type over all 36 order pairs and 3 dims: equal where the reference is sound; D1 cases
  equal the oracle run on the reinterpreted input; D2 / D3 cases differ;
- compute_deriv: equal to the oracle's reference-axis mode for every order (D7), and to the plain
  mode for the identity / transposition orders;
- D6 (plan cache ignores the r2r kind) on its characteristic cases;
- the 64^3 and 384x256x257 configurations at full size.
The defect labels D1-D7 are described in tests/refpin.py.  Skipped where the reference sources
are absent.
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import refpin as R

pyref = pytest.importorskip("pyref")
if not pyref.available():
    pytest.skip("reference sources not present (set P3DFFT_REFERENCE_DIR)", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def rel(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ref(oracle):
    pyref.lib()
    return pyref


# ---- the reference's own sample programs --------------------------------------------------
@pytest.mark.parametrize("sample", sorted(R.SAMPLES))
def test_reference_sample_against_reference_build(ref, tmp_path, sample):
    r = R.run_sample(sample, "ref", str(tmp_path))
    assert R.sample_passed(r, sample), r.stdout[-3000:] + r.stderr[-2000:]


# ---- 3D ------------------------------------------------------------------------------------
TYPESETS_3D = {
    "r2c_c2c_c2c": (R.R2C_D, R.C2C_FD, R.C2C_FD),
    "c2r_c2c_c2c": (R.C2R_D, R.C2C_BD, R.C2C_BD),
    "c2c_forward": (R.C2C_FD, R.C2C_FD, R.C2C_FD),
    "r2c_c2c_dct1": (R.R2C_D, R.C2C_FD, R.DCT1_CD),
    "real_dct2_dst2_dct3": (R.DCT2_RD, R.DST2_RD, R.DCT3_RD),
    "r2c_c2c_empty": (R.R2C_D, R.C2C_FD, R.EMPTY_DC),
    "r2c_single": (R.R2C_S, R.C2C_FS, R.C2C_FS),
}


def _x3(types, g1, mo1, seed):
    dt1 = R.dt_of(types[0])[0] if R.kind_of(types[0]) != 1 else 1
    cplx = not any(R.kind_of(t) == 1 for t in types) and any(R.dt_of(t)[0] == 2 for t in types)
    return R.seeded(R.storage_shape(g1, mo1), seed, cplx, R.prec_of(types[0]))


@pytest.mark.parametrize("name", sorted(TYPESETS_3D))
def test_3d_exec_equals_reference(ref, oracle, name):
    types = TYPESETS_3D[name]
    g1, dcs1, g2, dcs2 = R.grids_3d(types, (12, 10, 8))
    single = R.prec_of(types[0]) == 4
    worst = 0.0
    for mo1 in R.PERMS:
        for mo2 in R.PERMS:
            ref.reset()
            x = _x3(types, g1, mo1, 11)
            yr = ref.RefPlan3D(types, g1, mo1, g2, mo2, dcs1, dcs2).exec(x)
            yo = oracle.OraclePlan(types, g1, mo1, g2, mo2, dcs1, dcs2).exec(x)
            assert yr.shape == yo.shape, (mo1, mo2)
            worst = max(worst, rel(yr, yo))
    # same arithmetic on both sides: identical in FP64; the reference rounds FP32 stages
    assert worst <= (1e-6 if single else 1e-15), worst


def test_3d_exec_deriv_equals_reference_outside_defects(ref, oracle):
    gd = (12, 10, 8)
    counts = {"equal": 0, "D4": 0, "D5": 0}
    for types in [(R.R2C_D, R.C2C_FD, R.C2C_FD), (R.C2C_FD, R.C2C_FD, R.C2C_FD), (R.R2C_D, R.C2C_FD, R.DCT1_CD)]:
        g1, dcs1, g2, dcs2 = R.grids_3d(types, gd)
        for mo1 in R.PERMS:
            for mo2 in R.PERMS:
                o = oracle.OraclePlan(types, g1, mo1, g2, mo2, dcs1, dcs2)
                st = o.stages()
                for idir in range(3):
                    if R.d4_deriv_crash(st, idir):
                        counts["D4"] += 1
                        continue
                    ref.reset()
                    x = _x3(types, g1, mo1, 5 + idir)
                    e = rel(ref.RefPlan3D(types, g1, mo1, g2, mo2, dcs1, dcs2).exec(x, idir=idir), o.exec(x, idir=idir))
                    if R.d5_deriv_stage_defect(st, idir):
                        counts["D5"] += 1
                        continue
                    assert e <= 1e-15, (types, mo1, mo2, idir, e)
                    counts["equal"] += 1
    assert counts["equal"] >= 140 and counts["D4"] > 0 and counts["D5"] > 0, counts


def test_d5_reorder_deriv_branch_is_wrong_in_the_reference(ref, oracle):
    """One D5 case: the reference's derivative is not i*k times the spectrum."""
    types = (R.R2C_D, R.C2C_FD, R.C2C_FD)
    g1, dcs1, g2, dcs2 = R.grids_3d(types, (12, 10, 8))
    o = oracle.OraclePlan(types, g1, (0, 1, 2), g2, (0, 1, 2), dcs1, dcs2)
    assert R.d5_deriv_stage_defect(o.stages(), 1)
    ref.reset()
    x = _x3(types, g1, (0, 1, 2), 3)
    assert rel(ref.RefPlan3D(types, g1, (0, 1, 2), g2, (0, 1, 2), dcs1, dcs2).exec(x, idir=1), o.exec(x, idir=1)) > 1e-2


_D4_CHILD = r"""
import sys
sys.path[:0] = [{oracle!r}, {tests!r}]
import numpy as np, pyref, refpin as R
t = (R.R2C_D, R.C2C_FD, R.C2C_FD)
g1, d1, g2, d2 = R.grids_3d(t, (12, 10, 8))
p = pyref.RefPlan3D(t, g1, (0, 1, 2), g2, (0, 1, 2), d1, d2)
p.exec(R.seeded(R.storage_shape(g1, (0, 1, 2)), 1, False), idir=0)
print("returned")
"""


def test_d4_deriv_on_empty_stage_crashes_the_reference(ref, oracle):
    """The plan (0,1,2)->(0,1,2) ends with an EMPTY reorder stage along dim 0; the reference's
    exec_deriv(idir=0) calls its NULL derivative exec.  Run in a child process (CPU only)."""
    types = (R.R2C_D, R.C2C_FD, R.C2C_FD)
    g1, dcs1, g2, dcs2 = R.grids_3d(types, (12, 10, 8))
    assert R.d4_deriv_crash(oracle.OraclePlan(types, g1, (0, 1, 2), g2, (0, 1, 2), dcs1, dcs2).stages(), 0)
    code = _D4_CHILD.format(oracle=os.path.join(ROOT, "oracle"), tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "returned" not in r.stdout, (r.returncode, r.stdout[-500:])


# ---- 1D ------------------------------------------------------------------------------------
def test_1d_every_type_and_order_pair(ref, oracle):
    gd = (8, 6, 10)
    counts = {"sound": 0, "D1": 0, "D2": 0, "D3": 0}
    for tid in range(44):
        prec = R.prec_of(tid)
        tol = 1e-6 if prec == 4 else 1e-15
        for dim in range(3):
            g1, g2 = R.grids_1d(tid, dim, gd)
            for mo1 in R.PERMS:
                for mo2 in R.PERMS:
                    ref.reset()
                    x = R.seeded(R.storage_shape(g1, mo1), tid + 100 * dim, R.dt_of(tid)[0] == 2, prec)
                    yr = ref.RefPlan1D(tid, dim, g1, mo1, g2, mo2).exec(x)
                    if R.d1_reinterprets(tid, dim, mo1, mo2):
                        mq = R.swap0(mo1, dim)
                        yq = oracle.exec_stage(tid, dim, g1, mq, g2, mo2, x.reshape(R.storage_shape(g1, mq)))
                        assert rel(yr, yq) <= tol, ("D1", tid, dim, mo1, mo2)
                        counts["D1"] += 1
                        continue
                    yo = oracle.exec_stage(tid, dim, g1, mo1, g2, mo2, x)
                    e = rel(yr, yo)
                    if R.d2_half_copy(tid, dim, mo1, mo2):
                        assert e > 0.1, ("D2", tid, mo1, mo2, e)
                        counts["D2"] += 1
                    elif R.d3_reorder_out_021(tid, mo1, mo2):
                        assert e > 0.1, ("D3", tid, mo1, mo2, e)
                        counts["D3"] += 1
                    else:
                        assert e <= tol, (tid, dim, mo1, mo2, e)
                        counts["sound"] += 1
    assert counts["sound"] > 2000 and min(counts.values()) > 0, counts


# ---- compute_deriv -------------------------------------------------------------------------
def test_compute_deriv_reference_axis(ref, oracle):
    gd = (12, 10, 8)
    for mo in R.PERMS:
        involution = R.inv_mo(mo) == tuple(mo)
        for dcs in (-1, 0, 1, 2):
            g = list(gd)
            if dcs >= 0:
                g[dcs] = gd[dcs] // 2 + 1
            for idir in range(3):
                ref.reset()
                x = R.seeded(R.storage_shape(g, mo), 7 + idir, True)
                yr = ref.compute_deriv(x, g, mo, dcs, idir)
                assert np.array_equal(yr, oracle.compute_deriv(x, g, mo, dcs, idir, ref_axis=True)), (mo, dcs, idir)
                plain = oracle.compute_deriv(x, g, mo, dcs, idir)
                if involution:
                    assert np.array_equal(yr, plain)
                else:
                    assert rel(yr, plain) > 1e-2, (mo, dcs, idir)


# ---- D6 ------------------------------------------------------------------------------------
@pytest.mark.parametrize("types,mo2,effective", [
    ((R.DCT2_RD, R.DST2_RD, R.DCT2_RD), (0, 1, 2), (R.DCT2_RD, R.DCT2_RD, R.DCT2_RD)),
    ((R.DCT2_RD, R.DST2_RD, R.DCT3_RD), (0, 1, 2), (R.DCT2_RD, R.DCT3_RD, R.DCT3_RD)),
    ((R.DCT2_RD, R.DST2_RD, R.DCT3_RD), (1, 0, 2), (R.DCT2_RD, R.DCT2_RD, R.DCT3_RD)),
])
def test_d6_plan_cache_ignores_r2r_kind(ref, oracle, types, mo2, effective):
    """On an 8^3 grid the y stage (planned last) finds a cached r2r plan with its N, m and strides
    and runs that plan's kind: the reference's output is the oracle's for the substituted types."""
    gd = (8, 8, 8)
    ref.reset()
    x = R.seeded(gd, 1, False)
    yr = ref.RefPlan3D(types, gd, (0, 1, 2), gd, mo2).exec(x)
    assert rel(yr, oracle.OraclePlan(effective, gd, (0, 1, 2), gd, mo2).exec(x)) <= 1e-15
    assert rel(yr, oracle.OraclePlan(types, gd, (0, 1, 2), gd, mo2).exec(x)) > 1e-2


# ---- full-size configurations --------------------------------------------------------------
def test_config1_64cube_round_trip(ref, oracle):
    gd, g2 = (64, 64, 64), (33, 64, 64)
    fwd, bwd = (R.R2C_D, R.C2C_FD, R.C2C_FD), (R.C2R_D, R.C2C_BD, R.C2C_BD)
    ref.reset()
    x = R.seeded(R.storage_shape(gd, (0, 1, 2)), 64, False)
    yr = ref.RefPlan3D(fwd, gd, (0, 1, 2), g2, (1, 2, 0), -1, 0).exec(x)
    yo = oracle.OraclePlan(fwd, gd, (0, 1, 2), g2, (1, 2, 0), -1, 0).exec(x)
    assert rel(yr, yo) <= 1e-15
    zr = ref.RefPlan3D(bwd, g2, (1, 2, 0), gd, (0, 1, 2), 0, -1).exec(yr)
    assert rel(zr / np.prod(gd), x) <= 1e-14


def test_config3_mixed_types_full_size(ref, oracle):
    gd = (384, 256, 257)
    types = (R.R2C_D, R.C2C_FD, R.DCT1_CD)
    g1, dcs1, g2, dcs2 = R.grids_3d(types, gd)
    ref.reset()
    x = R.seeded(R.storage_shape(g1, (0, 1, 2)), 3, False)
    yr = ref.RefPlan3D(types, g1, (0, 1, 2), g2, (1, 2, 0), dcs1, dcs2).exec(x)
    yo = oracle.OraclePlan(types, g1, (0, 1, 2), g2, (1, 2, 0), dcs1, dcs2).exec(x)
    assert rel(yr, yo) <= 1e-15
