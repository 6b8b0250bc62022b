"""Shared fixtures.  CPU tests (`-m "not gpu"`) cover the oracle, the planner and the C-ABI
surface; GPU tests (`-m gpu`) compare the CUDA path, called through the C ABI, with the oracle."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "p3dfft.3_gb300")
for p in (os.path.join(ROOT, "oracle"), PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def p3d():
    import build_lib
    build_lib.build()
    import p3dfft_gb300
    p3dfft_gb300.lib()
    return p3dfft_gb300


@pytest.fixture(scope="session")
def gpu(p3d):
    """The library on a GPU; fails (does not skip) when the CUDA path cannot run.

    The oracle-parity tests compare against the transforms' defined results, so the session runs
    with the library's reference-compatibility mode off (compute_deriv along logical dim idir, 1D
    inputs read in their declared order); tests against the reference's own outputs
    (test_gpu_ref_golden.py) switch it on for their duration."""
    import ctypes
    p = p3d.lib().p3dfft_gb300_device_alloc(16)
    if not p:
        raise RuntimeError("CUDA device unavailable: " + p3d.lib().p3dfft_last_error_string().decode())
    p3d.lib().p3dfft_gb300_device_free(ctypes.c_void_p(p))
    p3d.set_reference_compat(False)
    return p3d


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


def seeded_field(shape, seed, dtype=np.float64):
    """U[-1,1) draws from numpy's PCG64 generator (seed recorded in each test)."""
    rng = np.random.default_rng(seed)
    if np.issubdtype(dtype, np.complexfloating):
        x = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    else:
        x = rng.uniform(-1, 1, shape)
    return np.ascontiguousarray(x.astype(dtype))
