"""GPU: batched execution of independent R2C -> C2R round trips (p3dfft_gb300_batch_*).

Every job's forward spectrum and round trip must be bit-identical to the same plan run alone
through p3dfft_gb300_exec3d with IEEE-double intermediate fields (the batch runs the same kernels,
only concurrently and from a CUDA graph), and the forward spectra must match the FP64 oracle (1e-12 for FP64 jobs, 1e-6 for FP32)."""
import numpy as np
import pytest

from conftest import rel_l2, seeded_field

pytestmark = pytest.mark.gpu

SHAPES = [(32, 32, 32), (24, 20, 18), (64, 48, 40), (40, 36, 30), (64, 64, 64), (16, 32, 8)]


def _plans(p3d, gd, prec):
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
    if prec == 8:
        ft = [p3d.R2CFFT_D, p3d.CFFT_FORWARD_D, p3d.CFFT_FORWARD_D]
        bt = [p3d.C2RFFT_D, p3d.CFFT_BACKWARD_D, p3d.CFFT_BACKWARD_D]
    else:
        ft = [p3d.R2CFFT_S, p3d.CFFT_FORWARD_S, p3d.CFFT_FORWARD_S]
        bt = [p3d.C2RFFT_S, p3d.CFFT_BACKWARD_S, p3d.CFFT_BACKWARD_S]
    f = p3d.Transform3D(ft, gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    b = p3d.Transform3D(bt, gd2, (1, 2, 0), gd, (0, 1, 2), 0, -1)
    return f, b


class Job:
    def __init__(self, p3d, gd, prec, seed, idir=-1):
        self.p3d = p3d
        self.gd, self.prec, self.idir = gd, prec, idir
        self.f, self.b = _plans(p3d, gd, prec)
        rdt = np.float64 if prec == 8 else np.float32
        self.x = seeded_field(p3d.storage_shape(gd, (0, 1, 2)), seed).astype(rdt)
        self.spec = np.empty(self.f.out_shape(), self.f.out_dtype())
        self.back = np.empty_like(self.x)
        self.d_x = p3d.DeviceArray(self.x.nbytes)
        self.d_s = p3d.DeviceArray(self.spec.nbytes)
        self.d_y = p3d.DeviceArray(self.x.nbytes)
        self.d_x.upload(self.x)

    def add_to(self, batch, job_id):
        batch.add(job_id, self.f, self.d_x, self.d_s, self.idir)
        batch.add(job_id, self.b, self.d_s, self.d_y)

    def download(self):
        return self.d_s.download(np.empty_like(self.spec)), self.d_y.download(np.empty_like(self.back))

    def alone(self):
        # batches pass IEEE-double intermediate fields between stages (float-float intermediates
        # are a plain-exec optimisation); the alone run does the same, so results compare bit for bit
        self.p3d.set_ff_intermediates(False)
        try:
            self.f.exec(self.d_x, self.d_s, idir=self.idir)
            self.b.exec(self.d_s, self.d_y)
        finally:
            self.p3d.set_ff_intermediates(True)
        return self.download()


def _jobs(p3d, n_each=1, idir=-1):
    jobs = []
    k = 0
    for gd in SHAPES:
        for prec in (8, 4):
            for _ in range(n_each):
                jobs.append(Job(p3d, gd, prec, seed=100 + k, idir=idir))
                k += 1
    return jobs


@pytest.mark.parametrize("graph,grouped", [(True, True), (False, True), (True, False), (False, False)])
def test_batch_bit_identical_to_alone_and_matches_oracle(gpu, oracle, graph, grouped):
    p3d = gpu
    p3d.set_fp64_arith(1)
    jobs = _jobs(p3d, n_each=2)  # two jobs per (grid, precision): cohorts of two
    alone = [j.alone() for j in jobs]
    for j in jobs:  # clear outputs so the batch must write them
        j.d_s.upload(np.zeros_like(j.spec))
        j.d_y.upload(np.zeros_like(j.back))
    batch = p3d.Batch(nbranches=4, graph=graph, grouped=grouped)
    for i, j in enumerate(jobs):
        j.add_to(batch, i)
    k0 = p3d.kernel_count()
    batch.exec()  # eager run (+ graph recording)
    k1 = p3d.kernel_count()
    stages = sum(len(j.f.stages()) + len(j.b.stages()) for j in jobs)
    assert batch.kernels() == k1 - k0
    if grouped:  # cohorts of two: one launch per stage on a specialised kernel, two otherwise
        assert 0 < batch.groups() and stages // 2 <= batch.kernels() < stages
    else:
        assert batch.kernels() == stages and batch.groups() == 0
    for j, (s0, y0) in zip(jobs, alone):
        s, y = j.download()
        assert np.array_equal(s, s0) and np.array_equal(y, y0)
    # second exec: graph replay (or eager again) on new inputs written in place
    for i, j in enumerate(jobs):
        j.x = seeded_field(j.x.shape, 900 + i).astype(j.x.dtype)
        j.d_x.upload(j.x)
    batch.exec()
    assert p3d.kernel_count() - k1 == batch.kernels()
    for j in jobs:
        s, y = j.download()
        ref = oracle.OraclePlan(j.f.types if j.prec == 8 else _d_types(p3d, j.f.types), j.gd, (0, 1, 2),
                                (j.gd[0] // 2 + 1, j.gd[1], j.gd[2]), (1, 2, 0), -1, 0).exec(j.x.astype(np.float64))
        tol = 1e-12 if j.prec == 8 else 1e-6
        assert rel_l2(s, ref) < tol, (j.gd, j.prec)
        assert rel_l2(y / np.prod(j.gd), j.x) < tol, (j.gd, j.prec)


def _d_types(p3d, types_s):
    return [t + 1 for t in types_s]  # _S and _D type IDs are adjacent


def test_batch_with_derivative_and_many_jobs_per_branch(gpu):
    """24 jobs on 3 branches (8 per branch, sharing one scratch set), forward with fused d/dx."""
    p3d = gpu
    jobs = _jobs(p3d, n_each=2, idir=0)
    alone = [j.alone() for j in jobs]
    batch = p3d.Batch(nbranches=3)
    for i, j in enumerate(jobs):
        j.add_to(batch, 10 * i + 7)  # arbitrary job ids
    batch.exec()
    batch.exec()
    for j, (s0, y0) in zip(jobs, alone):
        s, y = j.download()
        assert np.array_equal(s, s0) and np.array_equal(y, y0)


def test_batch_rerecords_after_arith_change_and_add(gpu):
    p3d = gpu
    p3d.set_fp64_arith(1)
    jobs = [Job(p3d, (32, 24, 16), 8, seed=5), Job(p3d, (48, 40, 32), 8, seed=6)]
    batch = p3d.Batch(nbranches=2)
    jobs[0].add_to(batch, 0)
    batch.exec()
    p3d.set_fp64_arith(0)
    batch.exec()  # native DFMA: re-recorded
    s_native, _ = jobs[0].download()
    p3d.set_fp64_arith(1)
    jobs[1].add_to(batch, 1)
    batch.exec()
    s_ff, _ = jobs[0].download()
    assert rel_l2(s_native, s_ff) < 1e-13
    s1, y1 = jobs[1].download()
    assert rel_l2(y1 / np.prod(jobs[1].gd), jobs[1].x) < 1e-12


def test_batch_rejects_host_pointers(gpu):
    p3d = gpu
    f, _ = _plans(p3d, (16, 16, 16), 8)
    x = np.zeros((16, 16, 16))
    y = np.zeros(f.out_shape(), np.complex128)
    batch = p3d.Batch()
    with pytest.raises(p3d.P3DFFTError, match="device pointers"):
        batch.add(0, f, x, y)


def test_work_list_batch_merges_uneven_jobs(gpu, oracle):
    """Work-list mode: each stage level runs one launch per kernel (arithmetic, kind, FFT length)
    over the tiles of every job that needs it, whatever the jobs' grids, so uneven jobs that share a
    line length share a launch (one CTA per (stage, tile) item).  Results are bit-identical to each
    job run alone."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    shapes = [(64, 32, 48), (64, 48, 32), (32, 64, 40), (48, 64, 64), (64, 64, 64), (40, 32, 64)]
    jobs = [Job(p3d, gd, prec, seed=300 + i) for i, gd in enumerate(shapes) for prec in (8, 4)]
    alone = [j.alone() for j in jobs]
    for j in jobs:
        j.d_s.upload(np.zeros_like(j.spec))
        j.d_y.upload(np.zeros_like(j.back))
    batch = p3d.Batch(nbranches=4, graph=True, grouped="list")
    for i, j in enumerate(jobs):
        j.add_to(batch, i)
    batch.exec()
    stages = sum(len(j.f.stages()) + len(j.b.stages()) for j in jobs)
    assert 0 < batch.groups() and batch.kernels() <= 0.75 * stages, (batch.kernels(), stages)
    for j, (s0, y0) in zip(jobs, alone):
        s, y = j.download()
        assert np.array_equal(s, s0) and np.array_equal(y, y0), (j.gd, j.prec)
    for i, j in enumerate(jobs):  # graph replay on new inputs
        j.x = seeded_field(j.x.shape, 700 + i).astype(j.x.dtype)
        j.d_x.upload(j.x)
    batch.exec()
    for j in jobs:
        s, _ = j.download()
        ref = oracle.OraclePlan(j.f.types if j.prec == 8 else _d_types(p3d, j.f.types), j.gd, (0, 1, 2),
                                (j.gd[0] // 2 + 1, j.gd[1], j.gd[2]), (1, 2, 0), -1, 0).exec(j.x.astype(np.float64))
        assert rel_l2(s, ref) < (1e-12 if j.prec == 8 else 1e-6), (j.gd, j.prec)
