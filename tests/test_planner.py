"""CPU: the library's 3D planner (no GPU needed to plan) against the oracle's restatement of
build/templ.C, over transform-type combinations and all 36 memory-order pairs."""
import itertools

import pytest

PERMS = list(itertools.permutations(range(3)))


def _stage_key(st):
    return [(s["type"], s["dim"], tuple(s["gdims1"]), tuple(s["mo1"]), s["dcs1"], tuple(s["gdims2"]),
             tuple(s["mo2"]), s["dcs2"]) for s in st]


TYPESETS = {
    "rcc": ("R2CFFT_D", "CFFT_FORWARD_D", "CFFT_FORWARD_D"),
    "ccc": ("CFFT_FORWARD_D", "CFFT_FORWARD_D", "CFFT_FORWARD_D"),
    "c_r2c_mid": ("CFFT_FORWARD_D", "R2CFFT_D", "CFFT_FORWARD_D"),
    "r2c_last": ("CFFT_FORWARD_S", "CFFT_FORWARD_S", "R2CFFT_S"),
    "rc_dct": ("R2CFFT_D", "CFFT_FORWARD_D", "DCT1_COMPLEX_D"),
    "empty_mid": ("R2CFFT_D", "EMPTY_TYPE_DOUBLE_COMPLEX", "CFFT_FORWARD_D"),
    "dct_real": ("DCT1_REAL_D", "DST2_REAL_D", "DCT3_REAL_D"),
}


@pytest.mark.parametrize("name", sorted(TYPESETS))
def test_forward_planner_matches_oracle(p3d, oracle, name):
    ids = [p3d.TYPE_IDS[t] for t in TYPESETS[name]]
    gd = [12, 10, 8]
    for mo1, mo2 in itertools.product(PERMS, PERMS):
        gd2 = list(gd)
        dcs2 = -1
        for i, t in enumerate(ids):
            ti = oracle.type_info(t)
            if ti["dt1"] < ti["dt2"]:
                gd2[i] = gd[i] // 2 + 1
                dcs2 = i
        op = oracle.OraclePlan(ids, gd, mo1, gd2, mo2, -1, dcs2)
        f = p3d.Transform3D(ids, gd, mo1, gd2, mo2, -1, dcs2)
        assert _stage_key(f.stages()) == _stage_key(op.stages()), (name, mo1, mo2)


@pytest.mark.parametrize("mo1", PERMS)
def test_backward_planner_matches_oracle(p3d, oracle, mo1):
    ids = [p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D]
    gd = [16, 6, 10]
    gd1 = [9, 6, 10]
    for mo2 in PERMS:
        op = oracle.OraclePlan(ids, gd1, mo1, gd, mo2, 0, -1)
        b = p3d.Transform3D(ids, gd1, mo1, gd, mo2, 0, -1)
        assert _stage_key(b.stages()) == _stage_key(op.stages()), (mo1, mo2)


def test_sample_plan_hand_trace(p3d):
    """The stage list traced by hand from templ.C for sample/C++/test3D_r2c.C (forward x,y,z
    with orders (0,1,2)->(1,0,2)->(1,2,0); backward y,z,x via (2,0,1),(2,1,0),(0,1,2))."""
    n = 64
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], (n, n, n), (0, 1, 2),
                        (n // 2 + 1, n, n), (1, 2, 0), -1, 0)
    st = f.stages()
    assert [s["dim"] for s in st] == [0, 1, 2]
    assert [s["mo2"] for s in st] == [(0, 1, 2), (1, 0, 2), (1, 2, 0)]
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], (n // 2 + 1, n, n), (1, 2, 0),
                        (n, n, n), (0, 1, 2), 0, -1)
    st = b.stages()
    assert [s["dim"] for s in st] == [1, 2, 0]
    assert [s["mo2"] for s in st] == [(2, 0, 1), (2, 1, 0), (0, 1, 2)]


def test_planner_rejects_bad_inputs(p3d):
    with pytest.raises(p3d.P3DFFTError):
        p3d.Transform3D([p3d.R2CFFT_D, p3d.R2CFFT_D, p3d.CFFT_FORWARD_D], (8, 8, 8), (0, 1, 2), (5, 5, 8),
                        (0, 1, 2), -1, 0)
    with pytest.raises(p3d.P3DFFTError):
        p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], (8, 8, 8), (0, 1, 1), (5, 8, 8),
                        (0, 1, 2), -1, 0)
    with pytest.raises(p3d.P3DFFTError):  # output dims that do not fit the transform
        p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], (8, 8, 8), (0, 1, 2), (8, 8, 8),
                        (0, 1, 2), -1, 0)
    with pytest.raises(p3d.P3DFFTError):
        p3d.Transform3D([99, 5, 9], (8, 8, 8), (0, 1, 2), (5, 8, 8), (0, 1, 2), -1, 0)


def _strides(gd, mo):
    return [int(__import__("numpy").prod([gd[j] for j in range(3) if mo[j] < mo[i]])) for i in range(3)]


def _side_cost(s, gd, L, t, esz):
    if s[L] == 1:
        c, cd = 1.0, L
    elif s[t] != 1:
        return 4.0
    else:
        c, cd = (1.4 if s[L] >= 16384 else 1.0), t
    return c + (0.15 if (gd[cd] * esz) % 128 else 0.0)


def _stage_cost(st, oracle):
    """Load + store cost with the kernel's tile-dim choice (by output stride when the input lines
    are contiguous, else by input stride)."""
    ti = oracle.type_info(st["type"])
    L = st["dim"]
    a, b = (L + 1) % 3, (L + 2) % 3
    s1, s2 = _strides(st["gdims1"], st["mo1"]), _strides(st["gdims2"], st["mo2"])
    t = (a if s2[a] <= s2[b] else b) if s1[L] == 1 else (a if s1[a] <= s1[b] else b)
    return (_side_cost(s1, st["gdims1"], L, t, ti["dt1"] * ti["prec"]) +
            _side_cost(s2, st["gdims2"], L, t, ti["dt2"] * ti["prec"]))


def _cost(stages, oracle):
    return sum(_stage_cost(s, oracle) for s in stages if oracle.type_info(s["type"])["kind"] != 0)


@pytest.mark.parametrize("name", sorted(TYPESETS))
def test_executed_schedule_is_an_equivalent_reordering(p3d, oracle, name):
    """The executor's schedule applies the same 1D transform to every dim, chains its grids from the
    plan's input grid to its output grid, keeps R2C first / C2R last, and is never costlier than
    the reference schedule under the access-cost model."""
    ids = [p3d.TYPE_IDS[t] for t in TYPESETS[name]]
    gd = [48, 40, 36]
    for mo1, mo2 in itertools.product(PERMS, PERMS):
        gd2, dcs2 = list(gd), -1
        for i, t in enumerate(ids):
            ti = oracle.type_info(t)
            if ti["dt1"] < ti["dt2"]:
                gd2[i], dcs2 = gd[i] // 2 + 1, i
        f = p3d.Transform3D(ids, gd, mo1, gd2, mo2, -1, dcs2)
        ref, ex = f.stages(), f.stages(executed=True)
        assert tuple(ex[0]["gdims1"]) == tuple(gd) and tuple(ex[0]["mo1"]) == tuple(mo1)
        assert tuple(ex[-1]["gdims2"]) == tuple(gd2) and tuple(ex[-1]["mo2"]) == tuple(mo2)
        for a, b in zip(ex, ex[1:]):
            assert (a["gdims2"], a["mo2"]) == (b["gdims1"], b["mo1"])
        nonempty = lambda st: sorted((s["dim"], s["type"]) for s in st if oracle.type_info(s["type"])["kind"] != 0)
        assert nonempty(ex) == nonempty(ref)
        dt = oracle.type_info(ex[0]["type"])["dt1"]
        for s in ex:  # data types chain
            ti = oracle.type_info(s["type"])
            assert ti["dt1"] == dt
            dt = ti["dt2"]
        assert _cost(ex, oracle) <= _cost(ref, oracle) + 1e-9


def test_headline_schedule_has_no_far_strided_stage(p3d, oracle):
    n = 512
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], (n, n, n), (0, 1, 2),
                        (n // 2 + 1, n, n), (1, 2, 0), -1, 0)
    b = p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], (n // 2 + 1, n, n), (1, 2, 0),
                        (n, n, n), (0, 1, 2), 0, -1)
    for plan in (f, b):
        for s in plan.stages(executed=True):
            assert _stage_cost(s, oracle) <= 2.15 + 1e-9, s  # no far-strided or uncoalesced side
