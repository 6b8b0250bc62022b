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
