"""GPU: the serving loop (p3dfft_gb300_server_*).

Jobs of mixed sizes, kinds (R2C / C2C) and precisions run forward -> d/dx -> backward.  Each job's
result must be bit-identical when it runs alone and when it runs inside a mix of concurrent jobs
(the same kernels on the same data; only the scheduling differs), and must match the CPU oracle's
forward + derivative + backward (1e-12 relative L2 for FP64, 1e-5 for FP32)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

MIX = [((32, 24, 20), "r2c", 8), ((48, 40, 36), "c2c", 4), ((64, 30, 18), "r2c", 4), ((20, 45, 27), "c2c", 8),
       ((96, 32, 40), "r2c", 8), ((50, 50, 50), "c2c", 8), ((36, 64, 25), "r2c", 4), ((128, 16, 24), "c2c", 4)]


def _types(kind, prec):
    if kind == "r2c":
        f, b = (5, 9, 9), (7, 11, 11)
    else:
        f, b = (9, 9, 9), (11, 11, 11)
    if prec == 4:
        f, b = tuple(t - 1 for t in f), tuple(t - 1 for t in b)
    return f, b


class SJob:
    def __init__(self, p3d, gd, kind, prec, seed):
        self.gd, self.kind, self.prec = gd, kind, prec
        tf, tb = _types(kind, prec)
        gd2 = (gd[0] // 2 + 1, gd[1], gd[2]) if kind == "r2c" else gd
        dcs = 0 if kind == "r2c" else -1
        self.f = p3d.Transform3D(tf, gd, (0, 1, 2), gd2, (1, 2, 0), -1, dcs)
        self.b = p3d.Transform3D(tb, gd2, (1, 2, 0), gd, (0, 1, 2), dcs, -1)
        rng = np.random.default_rng(seed)
        shape = p3d.storage_shape(gd, (0, 1, 2))
        x = rng.uniform(-1, 1, shape)
        if kind == "c2c":
            x = x + 1j * rng.uniform(-1, 1, shape)
        rdt = {("r2c", 8): np.float64, ("r2c", 4): np.float32, ("c2c", 8): np.complex128, ("c2c", 4): np.complex64}
        self.x = np.ascontiguousarray(x.astype(rdt[(kind, prec)]))
        self.pin_in = p3d.PinnedArray(self.x.shape, self.x.dtype)
        self.pin_in.array[...] = self.x
        self.pin_out = p3d.PinnedArray(self.x.shape, self.x.dtype)

    def result(self):
        return self.pin_out.array.copy()


def _oracle_round_trip(oracle, p3d, j):
    tf, tb = _types(j.kind, 8)
    gd = j.gd
    gd2 = (gd[0] // 2 + 1, gd[1], gd[2]) if j.kind == "r2c" else gd
    dcs = 0 if j.kind == "r2c" else -1
    x = j.x.astype(np.float64 if j.kind == "r2c" else np.complex128)
    spec = oracle.OraclePlan(tf, gd, (0, 1, 2), gd2, (1, 2, 0), -1, dcs).exec(x, idir=0)
    return oracle.OraclePlan(tb, gd2, (1, 2, 0), gd, (0, 1, 2), dcs, -1).exec(spec)


def test_serve_alone_equals_mix_and_oracle(gpu, oracle):
    p3d = gpu
    p3d.set_fp64_arith(1)
    jobs = [SJob(p3d, gd, kind, prec, seed=70 + i) for i, (gd, kind, prec) in enumerate(MIX)]
    # alone: one slot, one job at a time
    srv = p3d.Server(4 << 30, nslots=1)
    alone = []
    for j in jobs:
        jid = srv.submit(j.f, j.b, j.pin_in.array, j.pin_out.array, idir=0)
        assert srv.wait(jid)
        alone.append(j.result())
        j.pin_out.array[...] = 0
    srv.close()
    # the mix: every job submitted at once (twice over, so jobs overlap with copies of themselves)
    srv = p3d.Server(4 << 30, nslots=8)
    outs2 = [p3d.PinnedArray(j.x.shape, j.x.dtype) for j in jobs]
    ids = []
    for j, o2 in zip(jobs, outs2):
        ids.append(srv.submit(j.f, j.b, j.pin_in.array, j.pin_out.array, idir=0))
        ids.append(srv.submit(j.f, j.b, j.pin_in.array, o2.array, idir=0))
    assert srv.drain() == 0
    st = srv.stats()
    assert st["completed"] == len(ids) and st["failed"] == 0 and st["max_running"] > 1
    for j, o2, a in zip(jobs, outs2, alone):
        assert np.array_equal(j.result(), a) and np.array_equal(o2.array, a), (j.gd, j.kind, j.prec)
    for k, jid in enumerate(ids):
        rc, (ta, tadm, td) = srv.job_times(jid)
        assert rc == 0 and ta <= tadm <= td
    srv.close()
    for j, a in zip(jobs, alone):
        ref = _oracle_round_trip(oracle, p3d, j)
        tol = 1e-12 if j.prec == 8 else 1e-5
        assert rel_l2(a, ref) < tol, (j.gd, j.kind, j.prec)


def test_serve_budget_admission_and_trace_replay(gpu):
    """A budget that fits two jobs at a time: never more than two run, all complete; arrivals in the
    future are held until their time; a job larger than the budget fails alone."""
    p3d = gpu
    j = SJob(p3d, (64, 64, 64), "r2c", 8, seed=5)
    need = 8 * 64 ** 3 + 16 * 33 * 64 * 64 + 2 * 16 * 33 * 64 * 64
    srv = p3d.Server(int(2.5 * need), nslots=8)
    t0 = srv.clock() + 0.05
    outs = [p3d.PinnedArray(j.x.shape, j.x.dtype) for _ in range(6)]
    ids = [srv.submit(j.f, j.b, j.pin_in.array, o.array, idir=0, arrival=t0 + 0.01 * k) for k, o in enumerate(outs)]
    assert srv.drain() == 0
    st = srv.stats()
    assert st["max_running"] <= 2 and st["completed"] == 6 and st["peak_hbm_bytes"] <= 2.5 * need
    for k, jid in enumerate(ids):
        rc, (ta, tadm, td) = srv.job_times(jid)
        assert rc == 0 and abs(ta - (t0 + 0.01 * k)) < 1e-9 and tadm >= ta
    ref = outs[0].array.copy()
    for o in outs[1:]:
        assert np.array_equal(o.array, ref)
    srv.close()
    big = SJob(p3d, (128, 128, 128), "r2c", 8, seed=6)
    srv = p3d.Server(need, nslots=2)
    jid = srv.submit(big.f, big.b, big.pin_in.array, big.pin_out.array, idir=0)
    with pytest.raises(p3d.P3DFFTError, match="TOO_LARGE"):
        srv.wait(jid)
    srv.close()


def test_serve_device_resident_fields(gpu):
    """Inputs and outputs already in HBM (no host copies): same result as host-staged jobs."""
    p3d = gpu
    j = SJob(p3d, (40, 48, 36), "c2c", 8, seed=9)
    d_in, d_out = p3d.DeviceArray(j.x.nbytes), p3d.DeviceArray(j.x.nbytes)
    d_in.upload(j.x)
    srv = p3d.Server(1 << 30, nslots=2)
    a = srv.submit(j.f, j.b, d_in, d_out, idir=0)
    b = srv.submit(j.f, j.b, j.pin_in.array, j.pin_out.array, idir=0)
    assert srv.wait(a) and srv.wait(b)
    y = d_out.download(np.empty_like(j.x))
    assert np.array_equal(y, j.result())
    srv.close()


def test_serve_failures_leave_the_other_jobs_untouched(gpu):
    """Host-side failures in a mix of concurrent jobs: one job's device allocation fails (injected
    on the host, as if the pool had no room) and one job is malformed (its forward plan is destroyed
    while it waits).  Both fail with their own error; every other job completes with output
    bit-identical to its run alone, and the server keeps its budget accounting."""
    p3d = gpu
    p3d.set_fp64_arith(1)
    jobs = [SJob(p3d, gd, kind, prec, seed=90 + i) for i, (gd, kind, prec) in enumerate(MIX)]
    srv = p3d.Server(4 << 30, nslots=1)
    alone = []
    for j in jobs:
        assert srv.wait(srv.submit(j.f, j.b, j.pin_in.array, j.pin_out.array, idir=0))
        alone.append(j.result())
        j.pin_out.array[...] = 0
    srv.close()

    srv = p3d.Server(4 << 30, nslots=8)
    t0 = srv.clock() + 0.2  # arrivals held back until the failures are armed
    ids = [srv.submit(j.f, j.b, j.pin_in.array, j.pin_out.array, idir=0, arrival=t0) for j in jobs]
    victim_out = p3d.PinnedArray(jobs[2].x.shape, jobs[2].x.dtype)
    victim = srv.submit(jobs[2].f, jobs[2].b, jobs[2].pin_in.array, victim_out.array, idir=0, arrival=t0)
    srv.inject_alloc_failure(victim)
    bad = SJob(p3d, MIX[3][0], MIX[3][1], MIX[3][2], seed=93)
    malformed = srv.submit(bad.f, bad.b, bad.pin_in.array, bad.pin_out.array, idir=0, arrival=t0)
    p3d.lib().p3dfft_gb300_destroy3d(bad.f.handle)
    bad.f.handle = -1
    p3d.lib().p3dfft_clear_error()
    assert srv.drain() != 0
    st = srv.stats()
    assert st["failed"] == 2 and st["completed"] == len(jobs), st
    with pytest.raises(p3d.P3DFFTError, match="CUDA"):
        srv.wait(victim)
    with pytest.raises(p3d.P3DFFTError, match="BAD_ARG"):
        srv.wait(malformed)
    for j, a, jid in zip(jobs, alone, ids):
        assert srv.wait(jid)
        assert np.array_equal(j.result(), a), (j.gd, j.kind, j.prec)
    assert not np.any(victim_out.array)
    srv.close()
    p3d.lib().p3dfft_clear_error()
