"""GPU: the reference's own sample programs, compiled unchanged against include/ and linked with
libp3dfft_gb300.so, run on the GPU and pass their own checks ("Results are correct": analytic
spectra of sine waves, round trips to 1e-14 of the grid size, spectral derivatives, 1D cosine /
sine / R2C transforms, an EMPTY dim, user memory orders).  The same programs and inputs pass
against the reference built here (tests/test_ref_pin.py), so both libraries agree with the
samples' expectations.

The sample sources are the reference's (sample/C, sample/C++); the test runs where they are
available: $P3DFFT_REFERENCE_SAMPLES, or the reference tree, and skips otherwise.
"""
import pytest

import refpin as R

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(R.sample_dir() is None, reason="reference sample programs not present "
                                                   "(set P3DFFT_REFERENCE_SAMPLES)")
@pytest.mark.parametrize("sample", sorted(R.SAMPLES))
def test_reference_sample_runs_unchanged_on_gpu(gpu, tmp_path, sample):
    r = R.run_sample(sample, "gb300", str(tmp_path))
    assert R.sample_passed(r, sample), r.stdout[-3000:] + r.stderr[-2000:]
