"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on seeded inputs.

Tolerances: FP64 (native DFMA and float-float) <= 1e-12 relative L2 against the FP64 oracle, as
the reference's FFTW path is required to match; FP32 <= 1e-6 relative L2 against the FP64 oracle.
"""
import itertools

import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-6
PERMS = list(itertools.permutations(range(3)))


def _arith_modes(prec):
    return [0, 1] if prec == 8 else [0]


def _r2c_pair(p3d, gd, mo1=(0, 1, 2), mo2=(1, 2, 0), prec=8):
    s = "D" if prec == 8 else "S"
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    f = p3d.Transform3D([p3d.TYPE_IDS["R2CFFT_" + s], p3d.TYPE_IDS["CFFT_FORWARD_" + s],
                         p3d.TYPE_IDS["CFFT_FORWARD_" + s]], gd, mo1, gd2, mo2, -1, 0)
    b = p3d.Transform3D([p3d.TYPE_IDS["C2RFFT_" + s], p3d.TYPE_IDS["CFFT_BACKWARD_" + s],
                         p3d.TYPE_IDS["CFFT_BACKWARD_" + s]], gd2, mo2, gd, mo1, 0, -1)
    return f, b, gd2


@pytest.mark.parametrize("arith", [0, 1])
@pytest.mark.parametrize("gd", [(9, 15, 7), (17, 5, 11), (1, 4, 3), (3, 3, 3)])
def test_r2c_forward_odd_x(gpu, oracle, gd, arith):
    """Odd x lengths: forward only.  The reference planner sizes a C2R output as 2*(n-1)
    (templ.C:274-277), so a 3D plan back to an odd x length is rejected, as asserted here."""
    p3d = gpu
    p3d.set_fp64_arith(arith)
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    types = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=99)
    yo = oracle.OraclePlan(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x)
    assert rel_l2(f.exec(x), yo) < TOL64
    with pytest.raises(p3d.P3DFFTError):
        p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)


@pytest.mark.parametrize("arith", [0, 1])
@pytest.mark.parametrize("gd", [(64, 64, 64), (12, 10, 6), (30, 20, 24), (2, 3, 4), (18, 5, 11), (384, 4, 3)])
def test_r2c_forward_backward_fp64(gpu, oracle, gd, arith):
    p3d = gpu
    p3d.set_fp64_arith(arith)
    f, b, gd2 = _r2c_pair(p3d, gd)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=1234)
    y = f.exec(x)
    of = oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    yo = of.exec(x)
    assert rel_l2(y, yo) < TOL64
    z = b.exec(y) / np.prod(gd)
    assert rel_l2(z, x) < TOL64
    ob = oracle.OraclePlan(b.types, gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    zo = ob.exec(yo)
    assert rel_l2(b.exec(yo), zo) < TOL64


def test_sample_sine_known_answer(gpu):
    """sample/C++/test3D_r2c.C: spectrum of sin*sin*sin is +-0.125i at (+-1,+-1,+-1) after
    normalisation, within 1e-14*N/4 max-abs; round trip within 1e-14*Nglob/4."""
    p3d = gpu
    p3d.set_fp64_arith(0)
    n = 64
    f, b, gd2 = _r2c_pair(p3d, (n, n, n))
    t = np.arange(n) * 2 * np.pi / n
    x = np.ascontiguousarray(np.sin(t)[None, None, :] * np.sin(t)[None, :, None] * np.sin(t)[:, None, None])
    y = f.exec(x) / n ** 3
    # storage (y, x, z) for memory order (1,2,0): shape (Ny, Nx/2+1, Nz)
    ref = np.zeros_like(y)
    for (ky, kz) in itertools.product([1, n - 1], [1, n - 1]):
        sy = 1 if ky == 1 else -1
        sz = 1 if kz == 1 else -1
        # X(kx=1) = -i/2 per sine; product: (-i/2)^3 * sy * sz = 0.125i * sy * sz
        ref[ky, 1, kz] = 0.125j * sy * sz
    assert np.max(np.abs(y - ref)) < 1e-14 * n * 0.25
    z = b.exec(np.ascontiguousarray(y))
    assert np.max(np.abs(z - x)) < 1e-14 * n ** 3 * 0.25


@pytest.mark.parametrize("arith", [0, 1])
@pytest.mark.parametrize("idir", [0, 1, 2])
def test_fused_derivative(gpu, oracle, idir, arith):
    p3d = gpu
    p3d.set_fp64_arith(arith)
    gd = (16, 12, 10)
    f, b, gd2 = _r2c_pair(p3d, gd)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=77)
    y = f.exec_deriv(x, idir=idir)
    yo = oracle.OraclePlan(f.types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x, idir=idir)
    assert rel_l2(y, yo) < TOL64


def test_derivative_known_answer(gpu):
    """sample/C++/test_deriv.C: d/dx_i of the sine product equals the product with cos in dim i."""
    p3d = gpu
    p3d.set_fp64_arith(0)
    n = 32
    f, b, _ = _r2c_pair(p3d, (n, n, n))
    t = np.arange(n) * 2 * np.pi / n
    s, c = np.sin(t), np.cos(t)
    x = np.ascontiguousarray(s[None, None, :] * s[None, :, None] * s[:, None, None])
    for idir in range(3):
        y = f.exec_deriv(x, idir=idir) / n ** 3
        z = b.exec(np.ascontiguousarray(y))
        fac = [s, s, s]
        fac[idir] = c
        ref = fac[0][None, None, :] * fac[1][None, :, None] * fac[2][:, None, None]
        assert np.max(np.abs(z - ref)) < 1e-14 * n ** 3 * 0.25


@pytest.mark.parametrize("mo1,mo2", [((0, 1, 2), (0, 1, 2)), ((0, 1, 2), (2, 1, 0)), ((1, 0, 2), (0, 2, 1)),
                                     ((2, 0, 1), (1, 2, 0)), ((1, 2, 0), (2, 0, 1)), ((0, 2, 1), (1, 0, 2))])
def test_c2c_memory_orders(gpu, oracle, mo1, mo2):
    p3d = gpu
    p3d.set_fp64_arith(0)
    gd = (8, 6, 10)
    types = [p3d.CFFT_FORWARD_D] * 3
    f = p3d.Transform3D(types, gd, mo1, gd, mo2)
    x = seeded_field(p3d.storage_shape(gd, mo1), seed=5, dtype=np.complex128)
    y = f.exec(x)
    yo = oracle.OraclePlan(types, gd, mo1, gd, mo2).exec(x)
    assert rel_l2(y, yo) < TOL64
    st = f.stages()
    ost = oracle.OraclePlan(types, gd, mo1, gd, mo2).stages()
    assert [(s["type"], s["dim"], s["mo2"]) for s in st] == [(s["type"], s["dim"], s["mo2"]) for s in ost]


@pytest.mark.parametrize("mo1", PERMS)
def test_r2c_all_input_orders(gpu, oracle, mo1):
    p3d = gpu
    p3d.set_fp64_arith(0)
    gd = (10, 6, 8)
    for mo2 in PERMS:
        gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
        types = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
        f = p3d.Transform3D(types, gd, mo1, gd2, mo2, -1, 0)
        x = seeded_field(p3d.storage_shape(gd, mo1), seed=11)
        yo = oracle.OraclePlan(types, gd, mo1, gd2, mo2, -1, 0).exec(x)
        assert rel_l2(f.exec(x), yo) < TOL64, (mo1, mo2)


@pytest.mark.parametrize("arith", [0, 1])
def test_mixed_types_dct1(gpu, oracle, arith):
    """Config 3 shape family: x R2C, y C2C, z DCT-I (complex), small case."""
    p3d = gpu
    p3d.set_fp64_arith(arith)
    gd = (12, 8, 9)
    gd2 = (7, 8, 9)
    types = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.DCT1_COMPLEX_D]
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=3)
    yo = oracle.OraclePlan(types, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0).exec(x)
    assert rel_l2(f.exec(x), yo) < TOL64


@pytest.mark.parametrize("gd", [(16, 12, 10), (14, 9, 15)])
def test_fp32_forms(gpu, oracle, gd):
    p3d = gpu
    f, b, gd2 = _r2c_pair(p3d, gd, prec=4)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=9)
    x32 = x.astype(np.float32)
    y = f.exec(x32)
    assert y.dtype == np.complex64
    yo = oracle.OraclePlan([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], gd, (0, 1, 2), gd2, (1, 2, 0),
                           -1, 0).exec(x32.astype(np.float64))
    assert rel_l2(y, yo) < TOL32
    z = b.exec(y) / np.prod(gd)
    assert rel_l2(z, x32) < TOL32


# ---- 1D transplan API over every kind ----
KINDS_1D = ["CFFT_FORWARD", "CFFT_BACKWARD", "DCT1_REAL", "DST1_REAL", "DCT2_REAL", "DST2_REAL", "DCT3_REAL",
            "DST3_REAL", "DCT4_REAL", "DST4_REAL", "DCT1_COMPLEX", "DST1_COMPLEX", "DCT2_COMPLEX", "DST2_COMPLEX",
            "DCT3_COMPLEX", "DST3_COMPLEX", "DCT4_COMPLEX", "DST4_COMPLEX"]


@pytest.mark.parametrize("kind", KINDS_1D)
@pytest.mark.parametrize("n", [2, 5, 8, 13, 16, 24, 33])
@pytest.mark.parametrize("prec", [8, 4])
def test_1d_kinds(gpu, oracle, kind, n, prec):
    p3d = gpu
    p3d.set_fp64_arith(0)
    tid = p3d.TYPE_IDS[f"{kind}_{'D' if prec == 8 else 'S'}"]
    tid_d = p3d.TYPE_IDS[f"{kind}_D"]
    complex_data = kind.startswith("CFFT") or kind.endswith("COMPLEX")
    gd = (n, 3, 4)
    mo1, mo2 = (0, 1, 2), (0, 1, 2)
    dt = (np.complex128 if prec == 8 else np.complex64) if complex_data else (np.float64 if prec == 8 else np.float32)
    x = seeded_field(p3d.storage_shape(gd, mo1), seed=n, dtype=dt)
    if kind.startswith("DCT1") and n < 2:
        pytest.skip("DCT-I needs n > 1")
    tp = p3d.TransPlan(tid, gd, mo1, gd, mo2, 0)
    y = np.empty(p3d.storage_shape(gd, mo2), dt)
    tp.exec(x, y)
    yo = oracle.exec_stage(tid_d, 0, gd, mo1, gd, mo2, x.astype(np.complex128 if complex_data else np.float64))
    assert rel_l2(y, yo) < (TOL64 if prec == 8 else 5 * TOL32)


@pytest.mark.parametrize("dim", [0, 1, 2])
@pytest.mark.parametrize("mo1,mo2", [((0, 1, 2), (1, 0, 2)), ((2, 0, 1), (0, 1, 2)), ((1, 2, 0), (2, 1, 0))])
def test_1d_transplan_layouts(gpu, oracle, dim, mo1, mo2):
    p3d = gpu
    p3d.set_fp64_arith(0)
    gd = (6, 10, 4)
    gd2 = list(gd)
    gd2[dim] = gd[dim] // 2 + 1
    tp = p3d.TransPlan(p3d.R2CFFT_D, gd, mo1, gd2, mo2, dim)
    x = seeded_field(p3d.storage_shape(gd, mo1), seed=21)
    y = np.empty(p3d.storage_shape(gd2, mo2), np.complex128)
    tp.exec(x, y)
    yo = oracle.exec_stage(p3d.R2CFFT_D, dim, gd, mo1, gd2, mo2, x)
    assert rel_l2(y, yo) < TOL64


def test_in_place_c2c(gpu, oracle):
    """sample/C++/test3D_c2c_inplace.C: exec(AR, AR, true) on one buffer."""
    p3d = gpu
    p3d.set_fp64_arith(0)
    gd = (8, 8, 8)
    types = [p3d.CFFT_FORWARD_D] * 3
    f = p3d.Transform3D(types, gd, (0, 1, 2), gd, (0, 1, 2))
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=8, dtype=np.complex128)
    yo = oracle.OraclePlan(types, gd, (0, 1, 2), gd, (0, 1, 2)).exec(x)
    buf = x.copy()
    f.exec(buf, buf, OW=True)
    assert rel_l2(buf, yo) < TOL64


def test_device_pointers(gpu, oracle):
    torch = pytest.importorskip("torch")
    p3d = gpu
    p3d.set_fp64_arith(0)
    gd = (16, 8, 12)
    f, b, gd2 = _r2c_pair(p3d, gd)
    x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed=2)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(p3d.storage_shape(gd2, (1, 2, 0)), dtype=torch.complex128, device="cuda")
    f.exec(xd, yd)
    torch.cuda.synchronize()
    assert rel_l2(yd.cpu().numpy(), f.exec(x)) < 1e-15
    assert np.array_equal(xd.cpu().numpy(), x)  # OW=False leaves the input untouched


@pytest.mark.parametrize("mo", [(0, 1, 2), (1, 0, 2), (2, 1, 0), (1, 2, 0)])
@pytest.mark.parametrize("idir", [0, 1, 2])
def test_compute_deriv_standalone(gpu, oracle, mo, idir):
    p3d = gpu
    gd = (9, 8, 6)
    dcs = 0
    x = seeded_field(p3d.storage_shape(gd, mo), seed=4, dtype=np.complex128)
    y = np.empty_like(x)
    p3d.compute_deriv(x, y, gd, mo, dcs, idir)
    yo = oracle.compute_deriv(x, gd, mo, dcs, idir)
    assert rel_l2(y, yo) < 1e-15


def test_kernels_launch_counted(gpu):
    p3d = gpu
    p3d.lib().p3dfft_gb300_reset_kernel_count()
    f, b, gd2 = _r2c_pair(p3d, (8, 8, 8))
    f.exec(seeded_field((8, 8, 8), seed=1))
    assert p3d.kernel_count() == 3
