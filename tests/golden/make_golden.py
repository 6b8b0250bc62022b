"""Generates tests/golden/golden.npz: small seeded input/output pairs of the 3D pipeline.

Each case is computed by the CPU oracle and, independently, by scipy.fft applied along the
logical dimensions (R2C first, C2R last, DCT/DST via scipy's unnormalised types 1-4, which are
FFTW's REDFT/RODFT kinds), then written in the output memory order.  The script refuses to
write a fixture unless both agree to 1e-14 relative L2.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
import scipy.fft as sf

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402

# (name, types, gdims1, mo1, dcs1, gdims2, mo2, dcs2, idir, complex_input)
CASES = [
    ("r2c_sample_layout", (5, 9, 9), (8, 6, 4), (0, 1, 2), -1, (5, 6, 4), (1, 2, 0), 0, -1, False),
    ("r2c_deriv_z", (5, 9, 9), (8, 6, 4), (0, 1, 2), -1, (5, 6, 4), (1, 2, 0), 0, 2, False),
    ("r2c_deriv_x_odd", (5, 9, 9), (7, 6, 5), (0, 1, 2), -1, (4, 6, 5), (1, 2, 0), 0, 0, False),
    ("c2r_backward", (7, 11, 11), (5, 6, 4), (1, 2, 0), 0, (8, 6, 4), (0, 1, 2), -1, -1, True),
    ("mixed_r2c_c2c_dct1", (5, 9, 15), (6, 4, 5), (0, 1, 2), -1, (4, 4, 5), (1, 2, 0), 0, -1, False),
    ("c2c_orders", (9, 9, 9), (5, 6, 7), (2, 0, 1), -1, (5, 6, 7), (0, 2, 1), -1, -1, True),
    ("real_r2r_dct2_dst2_dct3", (21, 25, 29), (6, 5, 4), (1, 0, 2), -1, (6, 5, 4), (2, 1, 0), -1, -1, False),
    ("complex_dst1_dct4quirk_dst4", (19, 43, 39), (5, 4, 6), (0, 1, 2), -1, (5, 4, 6), (0, 1, 2), -1, -1, True),
]


def to_logical(a, gd, mo):
    """storage-order array -> array indexed [d0][d1][d2] by logical dimension"""
    a = np.asarray(a).reshape(pyoracle.storage_shape(gd, mo))
    # storage axis k (numpy axis) holds the logical dim with mo == 2-k
    axes = [0, 0, 0]
    for d in range(3):
        axes[d] = 2 - mo[d]
    return np.transpose(a, axes)


def to_storage(a, mo):
    perm = [0, 0, 0]
    for d in range(3):
        perm[2 - mo[d]] = d
    return np.ascontiguousarray(np.transpose(a, perm))


def scipy_apply(tid, a, d, n_out):
    info = pyoracle.type_info(tid)
    k = info["kind"]
    if k == pyoracle.K_EMPTY:
        return a
    if k == pyoracle.K_R2C:
        return sf.rfft(a, axis=d)
    if k == pyoracle.K_C2R:
        a = a.copy()
        idx = [slice(None)] * 3
        idx[d] = 0
        a[tuple(idx)] = a[tuple(idx)].real
        if n_out % 2 == 0:
            idx[d] = -1
            a[tuple(idx)] = a[tuple(idx)].real
        return sf.irfft(a, n=n_out, axis=d) * n_out
    if k == pyoracle.K_C2C_FWD:
        return sf.fft(a, axis=d)
    if k == pyoracle.K_C2C_BWD:
        return sf.ifft(a, axis=d) * a.shape[d]
    table = {pyoracle.REDFT00: ("dct", 1), pyoracle.REDFT10: ("dct", 2), pyoracle.REDFT01: ("dct", 3),
             pyoracle.REDFT11: ("dct", 4), pyoracle.RODFT00: ("dst", 1), pyoracle.RODFT10: ("dst", 2),
             pyoracle.RODFT01: ("dst", 3), pyoracle.RODFT11: ("dst", 4)}
    fam, t = table[info["r2r"]]
    f = getattr(sf, fam)
    if np.iscomplexobj(a):
        return f(a.real, type=t, axis=d) + 1j * f(a.imag, type=t, axis=d)
    return f(a, type=t, axis=d)


def deriv(a, d, r2c):
    M = a.shape[d]
    g = (M - 1) * 2 if r2c else M
    mid = g // 2
    k = np.arange(M, dtype=np.float64)
    k = np.where(k < mid, k, k - g)
    k[mid] = 0.0
    shp = [1, 1, 1]
    shp[d] = M
    return a * (1j * k.reshape(shp))


def scipy_reference(types, gd1, mo1, dcs1, gd2, mo2, dcs2, idir, x):
    plan = pyoracle.OraclePlan(types, gd1, mo1, gd2, mo2, dcs1, dcs2)
    a = to_logical(x, gd1, mo1)
    for st in plan.stages():
        d = st["dim"]
        a = scipy_apply(st["type"], a, d, st["gdims2"][d])
        if idir == d and pyoracle.type_info(st["type"])["dt2"] == 2 and pyoracle.type_info(st["type"])["kind"] != 0:
            a = deriv(a, d, pyoracle.type_info(st["type"])["kind"] == pyoracle.K_R2C)
    return to_storage(a, mo2)


def main():
    pyoracle.build()
    out = {}
    for i, (name, types, gd1, mo1, dcs1, gd2, mo2, dcs2, idir, cplx) in enumerate(CASES):
        rng = np.random.default_rng(1000 + i)
        shape = pyoracle.storage_shape(gd1, mo1)
        x = rng.uniform(-1, 1, shape)
        if cplx:
            x = x + 1j * rng.uniform(-1, 1, shape)
        y = pyoracle.OraclePlan(types, gd1, mo1, gd2, mo2, dcs1, dcs2).exec(x, idir=idir)
        ys = scipy_reference(types, gd1, mo1, dcs1, gd2, mo2, dcs2, idir, x)
        err = np.linalg.norm(y - ys) / np.linalg.norm(ys)
        print(f"{name:32s} oracle vs scipy rel L2 {err:.2e}")
        if err > 1e-14:
            raise SystemExit(f"{name}: oracle and scipy disagree ({err:.2e}); not writing fixtures")
        out[name + "__in"] = x
        out[name + "__out"] = y
        out[name + "__meta"] = np.array(list(types) + list(gd1) + list(mo1) + [dcs1] + list(gd2) + list(mo2) +
                                        [dcs2, idir], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"))


if __name__ == "__main__":
    main()
