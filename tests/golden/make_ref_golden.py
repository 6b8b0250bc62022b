"""Writes tests/golden/ref_golden.npz: outputs of the reference itself, for the GPU parity tests.

The reference is oracle/_ref/libp3dfft_ref.so: the reference's own build/*.C compiled unchanged by
oracle/build_ref.py, with FFTW's 1D arithmetic from oracle/refshim/fftw_shim.c (the oracle's).  It
runs only where the reference sources are (this script, not the GPU host), so its outputs travel
as fixtures.  Inputs are refpin.det_field (portable SplitMix64 fields) and are regenerated by the
tests from the stored seeds.  Cases (all FP64 unless named *_single):

  3d       7 type sets x 36 memory-order pairs on a 6x5x4 grid (full outputs)
  3d_deriv R2C/C2C/C2C exec_deriv, 36 pairs x 3 dims, where the reference is sound (not D4/D5)
  1d       every type ID 0..43: a leading-dim order pair and a D1 pair (full outputs)
  cderiv   compute_deriv, 6 memory orders x 3 dims x dim_conj_sym {-1, 0} (reference axis)
  config1  64^3 R2C/C2C/C2C forward, orders (0,1,2)->(1,2,0): refpin.fingerprint of the spectrum
  config3  384x256x257 R2C/C2C/DCT1-complex forward: fingerprint
  config2  512^3 R2C/C2C/C2C forward with the d/dz derivative fused: fingerprint

Defect labels (D1..D7) are described in tests/refpin.py.  Run:

    python tests/golden/make_ref_golden.py [--no-512]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
import pyoracle  # noqa: E402
import pyref  # noqa: E402
import refpin as R  # noqa: E402

OUT = os.path.join(HERE, "ref_golden.npz")
SMALL = (6, 5, 4)
SETS_3D = {
    "r2c_c2c_c2c": (R.R2C_D, R.C2C_FD, R.C2C_FD),
    "c2r_c2c_c2c": (R.C2R_D, R.C2C_BD, R.C2C_BD),
    "c2c_forward": (R.C2C_FD, R.C2C_FD, R.C2C_FD),
    "r2c_c2c_dct1": (R.R2C_D, R.C2C_FD, R.DCT1_CD),
    "real_dct2_dst2_dct3": (R.DCT2_RD, R.DST2_RD, R.DCT3_RD),
    "r2c_c2c_empty": (R.R2C_D, R.C2C_FD, R.EMPTY_DC),
    "r2c_single": (R.R2C_S, R.C2C_FS, R.C2C_FS),
}


def main():
    if not pyref.available():
        sys.exit("reference sources not present")
    pyoracle.build()
    arrays, metas = {}, []

    def add(meta, out):
        i = len(metas)
        meta = dict(meta)
        metas.append(meta)
        if isinstance(out, dict):
            for k, v in out.items():
                arrays[f"c{i}_{k}"] = np.asarray(v)
        else:
            arrays[f"c{i}"] = np.ascontiguousarray(out)

    seed = 1
    # ---- 3D exec on all memory-order pairs
    for name, types in SETS_3D.items():
        g1, dcs1, g2, dcs2 = R.grids_3d(types, SMALL)
        for mo1 in R.PERMS:
            for mo2 in R.PERMS:
                pyref.reset()
                x = R.det_field(R.storage_shape(g1, mo1), seed, R.input_is_complex(types), R.prec_of(types[0]))
                y = pyref.RefPlan3D(types, g1, mo1, g2, mo2, dcs1, dcs2).exec(x)
                add(dict(kind="3d", set=name, types=types, g1=g1, mo1=mo1, dcs1=dcs1, g2=g2, mo2=mo2, dcs2=dcs2,
                         idir=-1, seed=seed), y)
                seed += 1
    # ---- 3D exec_deriv where the reference is sound
    types = SETS_3D["r2c_c2c_c2c"]
    g1, dcs1, g2, dcs2 = R.grids_3d(types, SMALL)
    for mo1 in R.PERMS:
        for mo2 in R.PERMS:
            st = pyoracle.OraclePlan(types, g1, mo1, g2, mo2, dcs1, dcs2).stages()
            for idir in range(3):
                if R.d4_deriv_crash(st, idir) or R.d5_deriv_stage_defect(st, idir):
                    continue
                pyref.reset()
                x = R.det_field(R.storage_shape(g1, mo1), seed, False)
                y = pyref.RefPlan3D(types, g1, mo1, g2, mo2, dcs1, dcs2).exec(x, idir=idir)
                add(dict(kind="3d", set="r2c_deriv", types=types, g1=g1, mo1=mo1, dcs1=dcs1, g2=g2, mo2=mo2,
                         dcs2=dcs2, idir=idir, seed=seed), y)
                seed += 1
    # ---- 1D: every type, a leading pair and a D1 pair
    gd = (6, 4, 5)
    for tid in range(44):
        dim = tid % 3
        g1, g2 = R.grids_1d(tid, dim, gd)
        lead = tuple(R.swap0((0, 1, 2), dim))            # input leads with dim
        pairs = [(lead, R.PERMS[(tid * 5) % 6])]
        if R.kind_of(tid) != 0:
            nonlead = [m for m in R.PERMS if m[dim] != 0]
            pairs.append((nonlead[tid % len(nonlead)], nonlead[(tid + 1) % len(nonlead)]))
        for mo1, mo2 in pairs:
            if R.d2_half_copy(tid, dim, mo1, mo2) or R.d3_reorder_out_021(tid, mo1, mo2):
                continue
            pyref.reset()
            x = R.det_field(R.storage_shape(g1, mo1), seed, R.dt_of(tid)[0] == 2, R.prec_of(tid))
            y = pyref.RefPlan1D(tid, dim, g1, mo1, g2, mo2).exec(x)
            add(dict(kind="1d", type=tid, dim=dim, g1=g1, mo1=mo1, g2=g2, mo2=mo2,
                     d1=R.d1_reinterprets(tid, dim, mo1, mo2), seed=seed), y)
            seed += 1
    # ---- compute_deriv (reference axis)
    for mo in R.PERMS:
        for dcs in (-1, 0):
            g = list(SMALL)
            if dcs >= 0:
                g[dcs] = SMALL[dcs] // 2 + 1
            for idir in range(3):
                pyref.reset()
                x = R.det_field(R.storage_shape(g, mo), seed, True)
                add(dict(kind="cderiv", g=tuple(g), mo=mo, dcs=dcs, idir=idir, seed=seed),
                    pyref.compute_deriv(x, g, mo, dcs, idir))
                seed += 1
    # ---- full-size configurations (fingerprints)
    configs = [("config1", (64, 64, 64), SETS_3D["r2c_c2c_c2c"], -1, 641),
               ("config3", (384, 256, 257), SETS_3D["r2c_c2c_dct1"], -1, 643)]
    if "--no-512" not in sys.argv:
        configs.append(("config2", (512, 512, 512), SETS_3D["r2c_c2c_c2c"], 2, 642))
    for name, gdc, types, idir, cseed in configs:
        g1, dcs1, g2, dcs2 = R.grids_3d(types, gdc)
        mo1, mo2 = (0, 1, 2), (1, 2, 0)
        st = pyoracle.OraclePlan(types, g1, mo1, g2, mo2, dcs1, dcs2).stages()
        assert not (idir >= 0 and (R.d4_deriv_crash(st, idir) or R.d5_deriv_stage_defect(st, idir))), name
        t0 = time.time()
        pyref.reset()
        x = R.det_field(R.storage_shape(g1, mo1), cseed, False)
        y = pyref.RefPlan3D(types, g1, mo1, g2, mo2, dcs1, dcs2).exec(x, idir=idir)
        del x
        fp = R.fingerprint(y)
        del y
        add(dict(kind="config", name=name, types=types, g1=g1, mo1=mo1, dcs1=dcs1, g2=g2, mo2=mo2, dcs2=dcs2,
                 idir=idir, seed=cseed), fp)
        print(f"{name}: {time.time() - t0:.1f} s")
    arrays["meta"] = np.array(json.dumps(metas))
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(metas)} cases, {os.path.getsize(OUT) / 1e3:.0f} kB")


if __name__ == "__main__":
    main()
