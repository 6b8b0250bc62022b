"""CPU: host-side runtime pieces that need no GPU — the tuning-cache file format, plans the
library must refuse, and the batch, serving and tuning entry points failing loudly (not silently
computing on the CPU) without a device."""
import ctypes

import pytest


def test_tune_cache_file_round_trip(p3d, tmp_path):
    L = p3d.lib()
    src = tmp_path / "in.txt"
    src.write_text("# comment\n"
                   "3 0 8 1 2 2 0 64 48 40 64 48 40 1 64 3072 1 64 3072 | 1 0 0.012500\n"
                   "1 0 4 0 1 2 0 64 48 40 33 48 40 1 64 3072 1 33 1584 | 3 1 0.250000\n"
                   "malformed line without separator\n"
                   "1 0 4 0 1 2 0 8 8 8 5 8 8 1 8 64 1 5 40 | 9 0 1.0\n")
    p3d.tune_cache_clear()
    assert p3d.tune_cache_load(str(src)) == 2  # engine 9 is rejected
    out = tmp_path / "out.txt"
    p3d.tune_cache_save(str(out))
    rows = {}
    for line in out.read_text().splitlines():
        if not line.startswith("#"):
            key, val = line.split(" | ")
            e, t, ms = val.split()
            rows[key] = (int(e), int(t), float(ms))
    assert set(rows) == {"3 0 8 1 2 2 0 64 48 40 64 48 40 1 64 3072 1 64 3072",
                         "1 0 4 0 1 2 0 64 48 40 33 48 40 1 64 3072 1 33 1584"}
    assert rows["3 0 8 1 2 2 0 64 48 40 64 48 40 1 64 3072 1 64 3072"][:2] == (1, 0)
    assert abs(rows["1 0 4 0 1 2 0 64 48 40 33 48 40 1 64 3072 1 33 1584"][2] - 0.25) < 1e-7
    p3d.tune_cache_clear()
    with pytest.raises(p3d.P3DFFTError):
        p3d.tune_cache_load(str(tmp_path / "missing.txt"))


def test_runtimes_fail_loudly_without_device(p3d):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = p3d.lib()
    assert L.p3dfft_gb300_server_create(1 << 30, 4) == -1
    assert "device" in L.p3dfft_last_error_string().decode().lower()
    L.p3dfft_clear_error()
    b = L.p3dfft_gb300_batch_create(2)
    assert b >= 0
    assert L.p3dfft_gb300_batch_exec(b) in (0, 4)  # empty batch: nothing to run
    f = p3d.Transform3D([p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D], (8, 8, 8), (0, 1, 2), (5, 8, 8),
                        (1, 2, 0), -1, 0)
    assert L.p3dfft_gb300_autotune(f.handle, 0) == 4  # P3DFFT_ERR_NO_DEVICE
    assert L.p3dfft_gb300_preload_kernels() == 4
    L.p3dfft_clear_error()
    L.p3dfft_gb300_batch_destroy(b)


@pytest.mark.parametrize("bad", [(0, 4, 4), (4, 0, 4), (4, 4, -1)])
def test_empty_grid_is_rejected_at_plan_time(p3d, bad):
    with pytest.raises(p3d.P3DFFTError, match="BAD_ARG"):
        p3d.Transform3D([p3d.CFFT_FORWARD_D] * 3, bad, (0, 1, 2), bad, (0, 1, 2), -1, -1)


def test_c2r_to_real_length_one_is_rejected_at_plan_time(p3d):
    """A C2R from one complex point to one real point: the reference sizes the C2R output
    2(M-1) = 0 from M = 1 complex points (templ.C:274-277), a zero-length stage; the library
    refuses the plan, naming the mismatch."""
    with pytest.raises(p3d.P3DFFTError, match="PLAN"):
        p3d.Transform3D([p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D], (1, 4, 4), (0, 1, 2),
                        (1, 4, 4), (0, 1, 2), 0, -1)


def test_host_io_switches_round_trip(p3d, monkeypatch):
    """The host-I/O switches hold what they are set to: the link-stage CTA cap (-1 back to the
    default, which the environment variable overrides) and the host pipeline; the pageable switch
    reports "not on" without a device."""
    import torch
    monkeypatch.delenv("P3DFFT_GB300_LINK_CTAS", raising=False)
    try:
        p3d.set_link_ctas(37)
        assert p3d.get_link_ctas() == 37
        p3d.set_link_ctas(0)
        assert p3d.get_link_ctas() == 0
        p3d.set_link_ctas(-1)
        assert p3d.get_link_ctas() == -1
        monkeypatch.setenv("P3DFFT_GB300_LINK_CTAS", "200")
        assert p3d.get_link_ctas() == 200
        p3d.set_host_pipeline(False)
        assert p3d.get_host_pipeline() is False
    finally:
        p3d.set_link_ctas(-1)
        p3d.set_host_pipeline(True)
    if not torch.cuda.is_available():
        p3d.set_pageable_direct(True)
        try:
            assert p3d.get_pageable_direct() != 1
        finally:
            p3d.set_pageable_direct(False)
