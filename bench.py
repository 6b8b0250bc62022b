#!/usr/bin/env python3
"""Benchmark: 512^3 FP64 R2C -> (fused d/dz) -> C2R round trip of the P3DFFT++ pipeline.

One step = transform3D<double,complex_double>::exec_deriv (x R2C, y C2C, z C2C with the i*k_z
multiply fused into the z stage) followed by transform3D<complex_double,double>::exec (y C2C,
z C2C, x C2R), memory orders as in the reference sample test3D_r2c.C ((0,1,2) <-> (1,2,0)).

metric  GB/s of algorithmic traffic: the 3-pass pencil model, one HBM read + write per stage:
        round trip = 2*S_r + 10*S_c = 12,926,844,928 B at 512^3 FP64 (derivative adds 0).
value   device-resident buffers (inputs > L2, no flush needed), CUDA events on the library's
        stream, max over ranks.
e2e     same metric through the public C ABI with pinned HOST input and output buffers:
        H2D of the real field + forward + backward + D2H of the result inside the timed region.

--impl reference times the reference's CPU path for this workload on the host cores: the CPU
oracle (a plain-C restatement of the reference pipeline; FFTW and MPI, which the reference
needs, are absent on both machines) over a bounded sample of the same stages.
Multi-GPU: independent replicas (the path has no inter-GPU exchange on one rank's grid).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "p3dfft.3_gb300")
sys.path.insert(0, PKG)

N = int(os.environ.get("P3D_BENCH_N", "512"))
GD = tuple(int(v) for v in os.environ.get("P3D_BENCH_DIMS", f"{N},{N},{N}").split(","))
GD2 = (GD[0] // 2 + 1, GD[1], GD[2])
MO1, MO2 = (0, 1, 2), (1, 2, 0)
FWD = (5, 9, 9)    # R2CFFT_D, CFFT_FORWARD_D, CFFT_FORWARD_D
BWD = (7, 11, 11)  # C2RFFT_D, CFFT_BACKWARD_D, CFFT_BACKWARD_D
IDIR = 2           # d/dz, fused into the last forward stage
S_R = 8 * GD[0] * GD[1] * GD[2]
S_C = 16 * GD2[0] * GD2[1] * GD2[2]
ALG_BYTES = 2 * S_R + 10 * S_C
METRIC = "3D R2C+C2R GB/s (512^3 FP64 round trip with fused d/dz, 3-pass algorithmic bytes)"
WORKLOAD = f"{GD[0]}x{GD[1]}x{GD[2]} FP64 R2C/C2C/C2C + fused d/dz -> C2C/C2C/C2R round trip, memory orders (0,1,2)<->(1,2,0)"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Replicas:
    """Independent replicas, one process per GPU (the path has no inter-GPU exchange): a barrier
    and max-over-ranks timing through torch.distributed (NCCL on GPUs, gloo on CPU hosts)."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.torch = self.tdist = None
        self.dev = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as tdist
            use_cuda = torch.cuda.is_available()
            if use_cuda:
                torch.cuda.set_device(self.local)
                self.dev = "cuda"
            tdist.init_process_group("nccl" if use_cuda else "gloo")
            self.torch, self.tdist = torch, tdist

    def barrier(self):
        if self.tdist:
            if self.dev == "cuda":
                self.torch.cuda.synchronize()
            self.tdist.barrier()

    def _reduce(self, v, op):
        if not self.tdist:
            return v
        t = self.torch.tensor([float(v)], dtype=self.torch.float64, device=self.dev)
        self.tdist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        return self._reduce(v, self.tdist.ReduceOp.MAX if self.tdist else None)

    def sum(self, v):
        return self._reduce(v, self.tdist.ReduceOp.SUM if self.tdist else None)

    def close(self):
        if self.tdist:
            self.tdist.destroy_process_group()


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        rows = []
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------------------------------
def workload_config(world):
    """The workload both arms run (the GPU line and the CPU reference line carry the same dict)."""
    return {"workload": WORKLOAD, "grid": list(GD), "types_forward": "R2C_D,CFFT_FORWARD_D,CFFT_FORWARD_D",
            "types_backward": "C2R_D,CFFT_BACKWARD_D,CFFT_BACKWARD_D", "deriv": "d/dz fused",
            "l2": "inputs larger than L2 (1.07 GB real field, 1.08 GB spectrum); no flush",
            "input": "numpy PCG64 U[-1,1) seed 512+rank", "parallelism": f"replicas x{world}",
            "algorithmic_bytes_per_step": ALG_BYTES}


def run_reference(args, rank, world):
    """CPU reference arm: the oracle port of the reference path on all host cores."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    cores = os.cpu_count() or 1
    runners = []
    for types, g1, m1, d1, g2, m2, d2, idir in ((FWD, GD, MO1, -1, GD2, MO2, 0, IDIR),
                                                (BWD, GD2, MO2, 0, GD, MO1, -1, -1)):
        for st in pyoracle.OraclePlan(types, g1, m1, g2, m2, d1, d2).stages():
            run, b_in, b_out, nlines = pyoracle.stage_lines_runner(st, nthreads=cores)
            runners.append((run, b_in, b_out, nlines, st["dim"] == idir))
    # every line of every stage by default: each step is the whole round trip
    frac = float(os.environ.get("P3D_REF_SAMPLE", "1.0"))

    def step():
        nb = 0
        for run, b_in, b_out, nlines, deriv in runners:
            m = max(1, int(nlines * frac))
            run(0, m, deriv)
            nb += (b_in + b_out) * m / nlines
        return nb

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    nbytes = 0.0
    for _ in range(args.steps):
        nbytes += step()
    dt = time.perf_counter() - t0
    value = nbytes / dt / 1e9
    sample = (("all" if frac >= 1 else f"{frac:.4f} of the") +
              f" lines of each of the 6 stages of the {GD[0]}x{GD[1]}x{GD[2]} round trip per step "
              f"(oracle C port of the reference path, IEEE double, batched line engine: 16 lines per "
              f"vectorised Stockham FFT, OpenMP {cores} threads)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(world), "fp64_arith": "IEEE double (CPU)",
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(target_s=10.0):
    """Oracle port timed on whole round trips (every line of every stage, about target_s of CPU
    work in all), all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    cores = os.cpu_count() or 1
    runners = []
    for types, g1, m1, d1, g2, m2, d2, idir in ((FWD, GD, MO1, -1, GD2, MO2, 0, IDIR),
                                                (BWD, GD2, MO2, 0, GD, MO1, -1, -1)):
        for st in pyoracle.OraclePlan(types, g1, m1, g2, m2, d1, d2).stages():
            run, b_in, b_out, nlines = pyoracle.stage_lines_runner(st, nthreads=cores)
            runners.append((run, b_in + b_out, nlines, st["dim"] == idir))
    t0 = time.perf_counter()
    for run, _, nlines, deriv in runners:  # warm: one pass over every stage
        run(0, nlines, deriv)
    reps = max(3, int(target_s / max(time.perf_counter() - t0, 1e-3)))
    t0 = time.perf_counter()
    b_tot = 0.0
    for _ in range(reps):
        for run, nb, nlines, deriv in runners:
            run(0, nlines, deriv)
            b_tot += nb
    t_tot = time.perf_counter() - t0
    return {"value": b_tot / t_tot / 1e9, "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": f"{reps} whole {GD[0]}x{GD[1]}x{GD[2]} FP64 round trips, every line of the 6 stages "
                      f"(CPU oracle port of the reference path, batched line engine, OpenMP {cores} threads, "
                      f"{t_tot:.1f} s)"}


def load_traffic(kernel_key):
    """DRAM bytes per launch of a kernel at this workload, from a `TRAFFIC <kernel> <bytes>` line
    of a committed ncu summary under profiles/ (None when no summary covers it)."""
    pdir = os.path.join(ROOT, "profiles")
    try:
        for fn in sorted(os.listdir(pdir)):
            if not fn.endswith((".md", ".txt")):
                continue
            with open(os.path.join(pdir, fn)) as f:
                for line in f:
                    p = line.split()
                    if len(p) == 3 and p[0] == "TRAFFIC" and p[1] == kernel_key:
                        return int(p[2])
    except OSError:
        pass
    return None


def load_instr(kernel_key, tag="INSTR"):
    """Per-point count of a kernel from a `<tag> <kernel> <count>` line of a committed ncu summary
    under profiles/ (None when no summary covers it): INSTR = warp instructions, FP32OPS = FP32
    operations per complex FFT point."""
    pdir = os.path.join(ROOT, "profiles")
    try:
        for fn in sorted(os.listdir(pdir)):
            if not fn.endswith((".md", ".txt")):
                continue
            with open(os.path.join(pdir, fn)) as f:
                for line in f:
                    p = line.split()
                    if len(p) == 3 and p[0] == tag and p[1] == kernel_key:
                        return float(p[2])
    except OSError:
        pass
    return None


def _nfft(stage):
    kind = {5: 1, 7: 2}.get(stage["type"], 0)  # R2C_D, C2R_D, else C2C
    n = stage["gdims1"][stage["dim"]] if kind != 2 else stage["gdims2"][stage["dim"]]
    return kind, (n // 2 if kind else n)


def ff_variant(stages, i, arith, ff_on=True):
    """Float-float intermediate variant of stage i of a plan (bit 0: float-float input, bit 1:
    float-float output): the library links two consecutive float-float stages whose specialised
    kernels have float-float variants (C2C in / out, R2C out, C2R in; power-of-two FFT lengths
    64..2048)."""
    if not (arith and ff_on):
        return 0

    def capable(st):
        return st["type"] in (5, 7, 9, 11) and _nfft(st)[1] in (64, 128, 256, 512, 1024, 2048)

    def can_out(st):
        return capable(st) and st["type"] in (5, 9, 11)

    def can_in(st):
        return capable(st) and st["type"] in (7, 9, 11)

    v = 0
    if i > 0 and can_in(stages[i]) and can_out(stages[i - 1]):
        v |= 1
    if i + 1 < len(stages) and can_out(stages[i]) and can_in(stages[i + 1]):
        v |= 2
    return v


def kernel_id(stage, arith, n_dims, ff=0):
    """Name of the kernel instantiation that runs a stage (matches the ncu kernel names:
    k_fast<arithmetic, kind, FFT length, float-float variant>)."""
    kind, nfft = _nfft(stage)
    return f"k_fast<{'DFP' if arith else 'Native<double>'},{kind},{nfft},{ff}>"


# ------------------------------------------------------------------------------------------
# Batched uneven transforms: 48 independent R2C -> C2R round trips, sizes drawn from a seed among
# five grids, half FP32 and half FP64, run as one CUDA graph; against 48 sequential plain FP64 calls.
BATCH_SHAPES = [(64, 64, 64), (96, 128, 80), (128, 128, 128), (200, 200, 200), (256, 256, 256)]


def batch_jobs(n_jobs=48, seed=4):
    """(grid, precision) of each job: sizes uniform over BATCH_SHAPES, precisions a seeded
    permutation of n/2 FP32 and n/2 FP64."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(0, len(BATCH_SHAPES), n_jobs)
    precs = rng.permutation([4] * (n_jobs // 2) + [8] * (n_jobs - n_jobs // 2))
    return [(BATCH_SHAPES[s], int(p)) for s, p in zip(sizes, precs)]


def round_trip_bytes(gd, prec):
    """3-pass algorithmic bytes of one R2C -> C2R round trip: 2*S_r + 10*S_c."""
    s_r = prec * gd[0] * gd[1] * gd[2]
    s_c = 2 * prec * (gd[0] // 2 + 1) * gd[1] * gd[2]
    return 2 * s_r + 10 * s_c


def batch_workload(p3d, L, steps, warmup, nbranches=8, seed=4):
    """Times the batch (graph replay) and 48 sequential plain FP64 round trips; returns a dict."""
    import ctypes
    jobs = batch_jobs(seed=seed)
    plans = {}

    def plan_pair(gd, prec):
        key = (gd, prec)
        if key not in plans:
            gd2 = (gd[0] // 2 + 1, gd[1], gd[2])
            ft, bt = ((5, 9, 9), (7, 11, 11)) if prec == 8 else ((4, 8, 8), (6, 10, 10))
            plans[key] = (p3d.Transform3D(ft, gd, MO1, gd2, MO2, -1, 0), p3d.Transform3D(bt, gd2, MO2, gd, MO1, 0, -1))
        return plans[key]

    def buffers(gd, prec, seed_):
        n = gd[0] * gd[1] * gd[2]
        nc = (gd[0] // 2 + 1) * gd[1] * gd[2]
        d_x, d_s, d_y = p3d.DeviceArray(prec * n), p3d.DeviceArray(2 * prec * nc), p3d.DeviceArray(prec * n)
        x = np.random.default_rng(seed_).uniform(-1.0, 1.0, n)
        d_x.upload(x.astype(np.float64 if prec == 8 else np.float32))
        return d_x, d_s, d_y

    mixed = [(gd, prec, buffers(gd, prec, 4000 + i)) for i, (gd, prec) in enumerate(jobs)]
    plain = [(gd, 8, buffers(gd, 8, 4000 + i)) for i, (gd, _) in enumerate(jobs)]
    single = [(gd, 4, buffers(gd, 4, 4000 + i)) for i, (gd, _) in enumerate(jobs)]
    for gd, prec in set(jobs) | {(gd, p) for gd, _ in jobs for p in (4, 8)}:
        plan_pair(gd, prec)

    def make_batch(items, graph=True, grouped=True):
        bt = p3d.Batch(nbranches=nbranches, graph=graph, grouped=grouped)
        for j, (gd, prec, (d_x, d_s, d_y)) in enumerate(items):
            f, b = plan_pair(gd, prec)
            bt.add(j, f, d_x, d_s)
            bt.add(j, b, d_s, d_y)
        return bt

    def time_batch(bt):
        for _ in range(warmup):
            bt.exec()
        L.p3dfft_gb300_synchronize()
        k0 = p3d.kernel_count()
        L.p3dfft_gb300_event_record(4)
        for _ in range(steps):
            bt.exec()
        L.p3dfft_gb300_event_record(5)
        return L.p3dfft_gb300_event_elapsed_ms(4, 5) / steps, (p3d.kernel_count() - k0) // steps

    p3d.set_sync(False)
    # heuristic kernel choices first, then the autotuner's (per plan: every stage's engine and tile dim)
    b_heur = make_batch(mixed)
    ms_heur, _ = time_batch(b_heur)
    del b_heur
    t_tune = time.perf_counter()
    tuning = {}
    for (gd, prec), (f, b) in sorted(plans.items()):
        tf, tb = f.autotune(), b.autotune()
        tuning[f"{gd[0]}x{gd[1]}x{gd[2]}/{'fp64' if prec == 8 else 'fp32'}"] = {
            "forward": [[e, t, round(ms, 4)] for e, t, ms in tf], "backward": [[e, t, round(ms, 4)] for e, t, ms in tb]}
    t_tune = time.perf_counter() - t_tune
    b_mixed = make_batch(mixed)
    ms_mixed, k_mixed = time_batch(b_mixed)
    b_f64 = make_batch(plain)
    ms_b64, _ = time_batch(b_f64)
    b_f32 = make_batch(single)
    ms_b32, _ = time_batch(b_f32)
    # each FP32 job's result against the same job in FP64 (both unnormalised round trips)
    err32 = 0.0
    for (gd, _, (_, _, y32)), (_, _, (_, _, y64)) in zip(single, plain):
        a = y32.download(np.empty(gd[0] * gd[1] * gd[2], np.float32)).astype(np.float64)
        r = y64.download(np.empty(gd[0] * gd[1] * gd[2], np.float64))
        err32 = max(err32, float(np.linalg.norm(a - r) / np.linalg.norm(r)))
    b_nog = make_batch(mixed, graph=False)
    ms_nog, _ = time_batch(b_nog)
    b_br = make_batch(mixed, grouped=False)
    ms_br, k_br = time_batch(b_br)
    # work lists: one launch per (stage level, kernel) over all jobs' tiles
    b_wl = make_batch(mixed, grouped="list")
    ms_wl, k_wl = time_batch(b_wl)
    b_wl32 = make_batch(single, grouped="list")
    ms_wl32, _ = time_batch(b_wl32)

    # 48 sequential plain FP64 calls: the reference-style synchronous exec, one job after another
    p3d.set_sync(True)

    def sequential():
        for gd, prec, (d_x, d_s, d_y) in plain:
            f, b = plan_pair(gd, prec)
            p3d.check(L.p3dfft_gb300_exec3d(f.handle, ctypes.c_void_p(d_x.ptr), ctypes.c_void_p(d_s.ptr), -1, 0))
            p3d.check(L.p3dfft_gb300_exec3d(b.handle, ctypes.c_void_p(d_s.ptr), ctypes.c_void_p(d_y.ptr), -1, 0))

    for _ in range(max(1, warmup // 2)):
        sequential()
    n_seq = max(2, steps // 2)
    L.p3dfft_gb300_event_record(6)
    for _ in range(n_seq):
        sequential()
    L.p3dfft_gb300_event_record(7)
    ms_seq = L.p3dfft_gb300_event_elapsed_ms(6, 7) / n_seq
    p3d.set_sync(False)

    alg_mixed = sum(round_trip_bytes(gd, prec) for gd, prec in jobs)
    alg_plain = sum(round_trip_bytes(gd, 8) for gd, _ in jobs)
    n = len(jobs)
    hist = {}
    for gd, prec in jobs:
        k = f"{gd[0]}x{gd[1]}x{gd[2]}/{'fp64' if prec == 8 else 'fp32'}"
        hist[k] = hist.get(k, 0) + 1
    out = {
        "jobs": n, "seed": seed, "branches": nbranches, "mix": hist,
        "batch_graph_mixed": {"ms": ms_mixed, "round_trips_per_s": n / (ms_mixed * 1e-3),
                              "GB_per_s": alg_mixed / (ms_mixed * 1e-3) / 1e9, "kernels_per_exec": k_mixed,
                              "grouped_launches": b_mixed.groups(), "graph_launches_per_exec": 1,
                              "mode": "grouped: one launch per (cohort of same-plan jobs, stage) over all their tiles; cohorts on concurrent streams"},
        "batch_graph_branches_mixed": {"ms": ms_br, "round_trips_per_s": n / (ms_br * 1e-3), "kernels_per_exec": k_br,
                                       "mode": f"{nbranches} concurrent branch streams, one launch per stage"},
        "batch_graph_all_fp64": {"ms": ms_b64, "round_trips_per_s": n / (ms_b64 * 1e-3),
                                 "GB_per_s": alg_plain / (ms_b64 * 1e-3) / 1e9},
        "batch_graph_all_fp32": {"ms": ms_b32, "round_trips_per_s": n / (ms_b32 * 1e-3),
                                 "GB_per_s": alg_plain / 2 / (ms_b32 * 1e-3) / 1e9,
                                 "speedup_vs_sequential_fp64": ms_seq / ms_b32,
                                 "speedup_vs_batch_fp64": ms_b64 / ms_b32,
                                 "max_rel_l2_vs_fp64": err32},
        "batch_graph_work_list_mixed": {"ms": ms_wl, "round_trips_per_s": n / (ms_wl * 1e-3), "kernels_per_exec": k_wl,
                                        "work_list_launches": b_wl.groups(),
                                        "mode": "one launch per (stage level, kernel) over every job's tiles (device work list of (stage, tile) items); launches round-robin on the branch streams, each waiting only for the launches of its jobs' previous stage"},
        "batch_graph_work_list_all_fp32": {"ms": ms_wl32, "round_trips_per_s": n / (ms_wl32 * 1e-3),
                                           "speedup_vs_sequential_fp64": ms_seq / ms_wl32},
        "batch_streams_no_graph_mixed": {"ms": ms_nog, "round_trips_per_s": n / (ms_nog * 1e-3)},
        "sequential_plain_fp64": {"ms": ms_seq, "round_trips_per_s": n / (ms_seq * 1e-3),
                                  "GB_per_s": alg_plain / (ms_seq * 1e-3) / 1e9},
        "speedup_mixed_batch_vs_sequential_fp64": ms_seq / ms_mixed,
        "batch_graph_mixed_heuristic_kernels": {"ms": ms_heur, "round_trips_per_s": n / (ms_heur * 1e-3)},
        "autotune": {"seconds": t_tune, "engines": "1 specialised, 2 register, 3 generic; [engine, alt tile dim, ms]",
                     "choices": tuning},
    }
    for bt in (b_mixed, b_f64, b_f32, b_nog, b_br, b_wl, b_wl32):
        del bt
    return out


# ------------------------------------------------------------------------------------------
# Serving stream: Poisson arrivals of jobs with axes log-uniform in [32, 512] rounded to
# 2^a 3^b 5^c, 70/30 R2C/C2C, 60/40 FP32/FP64, each forward -> d/dx -> backward, admitted under a
# 120 GB HBM budget; latency percentiles at three arrival rates (fractions of the measured
# saturation throughput).  Fields are resident in HBM: each job copies its input from a device
# source field into its own pool-allocated field and its result out to a device sink.
def _smooth5_list():
    out = []
    for n in range(16, 1025):
        m = n
        for p in (2, 3, 5):
            while m % p == 0:
                m //= p
        if m == 1:
            out.append(n)
    return out


def serve_jobs(n_jobs, seed=5):
    """(dims, kind, prec) per job: each axis exp(U[ln 32, ln 512]) rounded to the nearest
    2^a 3^b 5^c (the R2C axis to the nearest even one, as C2R needs an even length)."""
    sm = np.array(_smooth5_list())
    even = sm[sm % 2 == 0]
    rng = np.random.default_rng(seed)
    raw = np.exp(rng.uniform(np.log(32), np.log(512), (n_jobs, 3)))
    kinds = np.where(rng.random(n_jobs) < 0.7, "r2c", "c2c")
    precs = np.where(rng.random(n_jobs) < 0.6, 4, 8)
    jobs = []
    for i in range(n_jobs):
        d = []
        for a in range(3):
            cand = even if (a == 0 and kinds[i] == "r2c") else sm
            d.append(int(cand[np.argmin(np.abs(cand - raw[i, a]))]))
        jobs.append((tuple(d), str(kinds[i]), int(precs[i])))
    return jobs


def serve_job_bytes(gd, kind, prec):
    """3-pass algorithmic bytes of one forward + backward (the fused derivative adds none)."""
    n = gd[0] * gd[1] * gd[2]
    if kind == "r2c":
        return round_trip_bytes(gd, prec)
    return 12 * 2 * prec * n


def mixed_types_workload(p3d, L, steps, arith):
    """384x256x257 with x R2C, y C2C, z DCT-I (complex), forward and backward, FP64 and FP32:
    per-stage device time (CUDA events between stages) and 3-pass GB/s of the round trip."""
    import ctypes
    gd, gd2 = (384, 256, 257), (193, 256, 257)
    out = {"grid": list(gd), "types_forward": "R2C,CFFT_FORWARD,DCT1_COMPLEX",
           "types_backward": "C2R,CFFT_BACKWARD,DCT1_COMPLEX"}
    for prec in (8, 4):
        sfx = "D" if prec == 8 else "S"
        ft = [p3d.TYPE_IDS[f"R2CFFT_{sfx}"], p3d.TYPE_IDS[f"CFFT_FORWARD_{sfx}"], p3d.TYPE_IDS[f"DCT1_COMPLEX_{sfx}"]]
        bt = [p3d.TYPE_IDS[f"C2RFFT_{sfx}"], p3d.TYPE_IDS[f"CFFT_BACKWARD_{sfx}"], p3d.TYPE_IDS[f"DCT1_COMPLEX_{sfx}"]]
        f = p3d.Transform3D(ft, gd, MO1, gd2, MO2, -1, 0)
        b = p3d.Transform3D(bt, gd2, MO2, gd, MO1, 0, -1)
        s_r = prec * gd[0] * gd[1] * gd[2]
        s_c = 2 * prec * gd2[0] * gd2[1] * gd2[2]
        d_x, d_s, d_y = p3d.DeviceArray(s_r), p3d.DeviceArray(s_c), p3d.DeviceArray(s_r)
        x = np.random.default_rng(384).uniform(-1.0, 1.0, gd[0] * gd[1] * gd[2])
        d_x.upload(x.astype(np.float64 if prec == 8 else np.float32))
        ms_f = (ctypes.c_double * 8)()
        ms_b = (ctypes.c_double * 8)()
        nf = L.p3dfft_gb300_profile_stages(f.handle, ctypes.c_void_p(d_x.ptr), ctypes.c_void_p(d_s.ptr), -1,
                                          max(5, steps), ms_f, 8)
        nb = L.p3dfft_gb300_profile_stages(b.handle, ctypes.c_void_p(d_s.ptr), ctypes.c_void_p(d_y.ptr), -1,
                                          max(5, steps), ms_b, 8)
        stages = []
        for plan, msv, n in ((f, ms_f, nf), (b, ms_b, nb)):
            for i, st in enumerate(plan.stages(executed=True)[:n]):
                stages.append({"dim": st["dim"], "type": st["type"], "ms": round(msv[i], 4)})
        ms = sum(st["ms"] for st in stages)
        alg = 2 * s_r + 10 * s_c
        key = ("fp64_float_float" if arith else "fp64_native") if prec == 8 else "fp32"
        out[key] = {"ms_per_round_trip": ms, "GB_per_s": alg / (ms * 1e-3) / 1e9, "stages": stages}
        del d_x, d_s, d_y, f, b
    return out


def serve_workload(p3d, n_jobs=10000, seed=5, fractions=(0.5, 0.75, 0.9), nslots=16, budget=120 << 30):
    jobs = serve_jobs(n_jobs, seed)
    plans = {}

    def plan_pair(gd, kind, prec):
        key = (gd, kind, prec)
        if key not in plans:
            if kind == "r2c":
                ft, bt, gd2, dcs = (5, 9, 9), (7, 11, 11), (gd[0] // 2 + 1, gd[1], gd[2]), 0
            else:
                ft, bt, gd2, dcs = (9, 9, 9), (11, 11, 11), gd, -1
            if prec == 4:
                ft, bt = tuple(t - 1 for t in ft), tuple(t - 1 for t in bt)
            plans[key] = (p3d.Transform3D(ft, gd, MO1, gd2, MO2, -1, dcs), p3d.Transform3D(bt, gd2, MO2, gd, MO1, dcs, -1))
        return plans[key]

    t_plan = time.perf_counter()
    pairs = [plan_pair(*j) for j in jobs]
    t_plan = time.perf_counter() - t_plan
    print(f"serve: {len(plans)} plans in {t_plan:.1f} s", file=sys.stderr, flush=True)
    maxn = 512 ** 3
    src, sink = {}, {}
    for prec in (4, 8):
        rdt = np.float32 if prec == 4 else np.float64
        x = np.random.default_rng(55 + prec).uniform(-1, 1, 2 * maxn).astype(rdt)
        src[prec] = p3d.DeviceArray(x.nbytes)
        src[prec].upload(x)
        sink[prec] = p3d.DeviceArray(x.nbytes)
        del x
    alg = np.array([serve_job_bytes(*j) for j in jobs], dtype=np.float64)

    def run(arrivals, srv):
        ids = []
        for (gd, kind, prec), (f, b), ta in zip(jobs, pairs, arrivals):
            ids.append(srv.submit(f, b, src[prec], sink[prec], idir=0, arrival=ta))
        srv.drain()
        t = np.array([srv.job_times(i)[1] for i in ids])
        return t[:, 0], t[:, 1], t[:, 2], srv.stats()

    out = {"jobs": n_jobs, "seed": seed, "slots": nslots, "budget_bytes": budget,
           "mix": {"r2c": sum(j[1] == "r2c" for j in jobs), "c2c": sum(j[1] == "c2c" for j in jobs),
                   "fp32": sum(j[2] == 4 for j in jobs), "fp64": sum(j[2] == 8 for j in jobs)},
           "distinct_grids": len(plans), "plan_time_s": t_plan,
           "mean_input_MB": float(np.mean([np.prod(j[0]) * j[2] * (1 if j[1] == "r2c" else 2) for j in jobs]) / 1e6)}
    # warm-up + saturation throughput: a closed burst of every job at once
    srv = p3d.Server(budget, nslots)
    lead = 0.3 + 1e-4 * n_jobs
    t0 = srv.clock() + lead
    ta, tadm, td, st = run([t0] * n_jobs, srv)
    srv.close()
    makespan = td.max() - t0
    cap = n_jobs / makespan
    print(f"serve: saturation {cap:.0f} jobs/s", file=sys.stderr, flush=True)
    out["saturation"] = {"jobs_per_s": cap, "GB_per_s": alg.sum() / makespan / 1e9,
                         "max_running": st["max_running"], "peak_hbm_GB": st["peak_hbm_bytes"] / 1e9,
                         "dispatcher_us_per_job": {"queue_work": st["host_launch_s"] / n_jobs * 1e6,
                                                   "release": st["host_release_s"] / n_jobs * 1e6}}
    rng = np.random.default_rng(seed + 1)
    out["rates"] = []
    for frac in fractions:
        rate = frac * cap
        srv = p3d.Server(budget, nslots)
        t0 = srv.clock() + lead
        arr = t0 + np.cumsum(rng.exponential(1.0 / rate, n_jobs))
        ta, tadm, td, st = run(arr, srv)
        srv.close()
        lat = (td - ta) * 1e3
        wait = (tadm - ta) * 1e3
        span = td.max() - ta.min()
        out["rates"].append({
            "offered_jobs_per_s": rate, "fraction_of_saturation": frac,
            "throughput_jobs_per_s": n_jobs / span, "GB_per_s": alg.sum() / span / 1e9,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                           "p99": float(np.percentile(lat, 99)), "max": float(lat.max()), "mean": float(lat.mean())},
            "queue_wait_ms": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99))},
            "failed": st["failed"], "max_running": st["max_running"], "peak_hbm_GB": st["peak_hbm_bytes"] / 1e9})
    del src, sink
    return out


def fp32_line_errors(p3d, lengths=(64, 128, 256, 512, 1024, 2048)):
    """FP32 C2C lines (64 x 16 of each length, U[-1,1) complex) against numpy's FP64 FFT of the
    same FP32 inputs: relative L2 error with split and with plain twiddles."""
    out = {}
    rng = np.random.default_rng(32)
    for n in lengths:
        g = (n, 64, 16)
        x = (rng.uniform(-1, 1, (16, 64, n)) + 1j * rng.uniform(-1, 1, (16, 64, n))).astype(np.complex64)
        ref = np.fft.fft(x.astype(np.complex128), axis=-1)
        row = {}
        for split in (True, False):
            p3d.set_fp32_split_twiddles(split)
            y = np.empty_like(x)
            p3d.TransPlan(p3d.CFFT_FORWARD_S, g, (0, 1, 2), g, (0, 1, 2), 0).exec(x, y)
            row["split" if split else "plain"] = float(np.linalg.norm(y - ref) / np.linalg.norm(ref))
        out[str(n)] = row
    p3d.set_fp32_split_twiddles(True)
    return out


def full_size_parity(p3d, f, b, d_in, d_spec, d_out):
    """The headline plans at full size against the reference: the forward transform with the
    fused d/dz derivative of the 512^3 reference input (tests/golden/ref_golden.npz, written from
    the reference's own build; compared by the size-independent fingerprint of tests/refpin.py),
    and the normalised plain round trip of the same input."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import refpin
    z = np.load(os.path.join(ROOT, "tests", "golden", "ref_golden.npz"))
    metas = json.loads(str(z["meta"]))
    hit = [(i, m) for i, m in enumerate(metas) if m["kind"] == "config" and m["name"] == "config2"]
    if not hit or tuple(hit[0][1]["g1"]) != GD:
        return {"skipped": "no 512^3 reference fixture for this grid"}
    i, m = hit[0]
    x = refpin.det_field(p3d.storage_shape(GD, MO1), m["seed"], False)
    d_in.upload(x)
    p3d.set_sync(True)
    f.exec(d_in, d_spec, idir=m["idir"])
    spec = d_spec.download(np.empty(p3d.storage_shape(GD2, MO2), np.complex128))
    ref = {k: z[f"c{i}_{k}"] for k in ("idx", "val", "proj", "norm")}
    err_ref = float(refpin.fingerprint_error(refpin.fingerprint(spec), ref))
    del spec
    f.exec(d_in, d_spec)
    b.exec(d_spec, d_out)
    back = d_out.download(np.empty(p3d.storage_shape(GD, MO1), np.float64)) / float(np.prod(GD))
    err_rt = float(np.linalg.norm(back - x) / np.linalg.norm(x))
    p3d.set_sync(False)
    return {"forward_ddz_vs_reference_fingerprint": err_ref, "normalised_round_trip_rel_l2": err_rt,
            "tolerance": 1e-12, "input": "refpin.det_field seed %d (the reference's 512^3 fixture input)" % m["seed"],
            "reference": "reference build/*.C compiled unchanged, outputs in tests/golden/ref_golden.npz"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arith", default="auto", choices=["auto", "df", "native"],
                    help="FP64 arithmetic: float-float (df) or native DFMA; auto = df")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="roundtrip", choices=["roundtrip", "batch", "serve"],
                    help="roundtrip: the 512^3 headline; batch: 48 uneven round trips; serve: the serving stream")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-workload summary")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-stream summary")
    ap.add_argument("--serve-jobs", type=int, default=10000)
    ap.add_argument("--serve-slots", type=int, default=16)
    ap.add_argument("--kernels-only", choices=["fp64", "fp32"], default=None,
                    help="run only the device-resident round trip of that form (profiling runs)")
    ap.add_argument("--e2e-only", choices=["fp64", "fp32"], default=None,
                    help="run only the round trip of that form from and to page-locked host arrays "
                         "(profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "batch":
        import p3dfft_gb300 as p3d
        import build_lib
        build_lib.build()
        res = batch_workload(p3d, p3d.lib(), args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({"workload": "batched uneven round trips", **res}), flush=True)
        return
    if args.e2e_only:
        import ctypes
        import p3dfft_gb300 as p3d
        import build_lib
        build_lib.build()
        L = p3d.lib()
        prec = 8 if args.e2e_only == "fp64" else 4
        rdt = np.float64 if prec == 8 else np.float32
        ft, bt = (FWD, BWD) if prec == 8 else (tuple(t - 1 for t in FWD), tuple(t - 1 for t in BWD))
        f = p3d.Transform3D(ft, GD, MO1, GD2, MO2, -1, 0)
        b = p3d.Transform3D(bt, GD2, MO2, GD, MO1, 0, -1)
        hin = p3d.PinnedArray(p3d.storage_shape(GD, MO1), rdt)
        hout = p3d.PinnedArray(p3d.storage_shape(GD, MO1), rdt)
        hin.array[...] = np.random.default_rng(512).uniform(-1.0, 1.0, hin.array.shape)
        d_spec = p3d.DeviceArray(S_C * prec // 8)
        vp = ctypes.c_void_p
        for k in range(args.warmup + args.steps):
            if k == args.warmup:
                L.p3dfft_gb300_synchronize()
                t0 = time.perf_counter()
            p3d.check(L.p3dfft_gb300_exec3d(f.handle, vp(hin.ptr), vp(d_spec.ptr), IDIR, 0))
            p3d.check(L.p3dfft_gb300_exec3d(b.handle, vp(d_spec.ptr), vp(hout.ptr), -1, 0))
        L.p3dfft_gb300_synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps)
        print(json.dumps({"e2e_only": args.e2e_only, "grid": list(GD), "ms_per_round_trip": ms}), flush=True)
        return
    if args.kernels_only:
        import ctypes
        import p3dfft_gb300 as p3d
        import build_lib
        build_lib.build()
        L = p3d.lib()
        p3d.set_fp64_arith(0 if args.arith == "native" else 1)
        prec = 8 if args.kernels_only == "fp64" else 4
        ft, bt = (FWD, BWD) if prec == 8 else (tuple(t - 1 for t in FWD), tuple(t - 1 for t in BWD))
        f = p3d.Transform3D(ft, GD, MO1, GD2, MO2, -1, 0)
        b = p3d.Transform3D(bt, GD2, MO2, GD, MO1, 0, -1)
        d_in, d_spec, d_out = p3d.DeviceArray(S_R * prec // 8), p3d.DeviceArray(S_C * prec // 8), p3d.DeviceArray(S_R * prec // 8)
        x = np.random.default_rng(512).uniform(-1.0, 1.0, p3d.storage_shape(GD, MO1))
        d_in.upload(x.astype(np.float64 if prec == 8 else np.float32))
        p3d.set_sync(False)
        vp = ctypes.c_void_p
        for k in range(args.warmup + args.steps):
            if k == args.warmup:
                L.p3dfft_gb300_synchronize()
                L.p3dfft_gb300_event_record(0)
            p3d.check(L.p3dfft_gb300_exec3d(f.handle, vp(d_in.ptr), vp(d_spec.ptr), IDIR, 0))
            p3d.check(L.p3dfft_gb300_exec3d(b.handle, vp(d_spec.ptr), vp(d_out.ptr), -1, 0))
        L.p3dfft_gb300_event_record(1)
        ms = L.p3dfft_gb300_event_elapsed_ms(0, 1) / max(1, args.steps)
        print(json.dumps({"kernels_only": args.kernels_only, "grid": list(GD), "ms_per_round_trip": ms,
                          "GB_per_s": ALG_BYTES * prec // 8 / (ms * 1e-3) / 1e9}), flush=True)
        return
    if args.workload == "serve":
        import p3dfft_gb300 as p3d
        import build_lib
        build_lib.build()
        res = serve_workload(p3d, n_jobs=args.serve_jobs, nslots=args.serve_slots)
        if rank == 0:
            print(json.dumps({"workload": "serving stream", **res}), flush=True)
        return

    import ctypes

    import p3dfft_gb300 as p3d
    import build_lib
    build_lib.build()
    L = p3d.lib()
    reps = Replicas()

    arith = 0 if args.arith == "native" else 1
    p3d.set_fp64_arith(arith)
    f = p3d.Transform3D(FWD, GD, MO1, GD2, MO2, -1, 0)
    b = p3d.Transform3D(BWD, GD2, MO2, GD, MO1, 0, -1)
    x = np.random.default_rng(512 + rank).uniform(-1.0, 1.0, p3d.storage_shape(GD, MO1))
    d_in = p3d.DeviceArray(S_R)
    d_spec = p3d.DeviceArray(S_C)
    d_out = p3d.DeviceArray(S_R)
    d_in.upload(x)

    def step(fin, fout):
        p3d.check(L.p3dfft_gb300_exec3d(f.handle, ctypes.c_void_p(fin), ctypes.c_void_p(d_spec.ptr), IDIR, 0))
        p3d.check(L.p3dfft_gb300_exec3d(b.handle, ctypes.c_void_p(d_spec.ptr), ctypes.c_void_p(fout), -1, 0))

    barrier = reps.barrier
    max_over_ranks = reps.max

    # ---- device-resident timed region ----
    p3d.set_sync(False)
    for _ in range(args.warmup):
        step(d_in.ptr, d_out.ptr)
    L.p3dfft_gb300_synchronize()
    barrier()
    k0 = p3d.kernel_count()
    with ClockSampler(local) as clk:
        L.p3dfft_gb300_synchronize()
        L.p3dfft_gb300_event_record(0)
        for _ in range(args.steps):
            step(d_in.ptr, d_out.ptr)
        L.p3dfft_gb300_event_record(1)
        ms = L.p3dfft_gb300_event_elapsed_ms(0, 1)
        L.p3dfft_gb300_synchronize()
    launches = p3d.kernel_count() - k0
    barrier()
    ms_step = max_over_ranks(ms / args.steps)
    value = ALG_BYTES * world / (ms_step * 1e-3) / 1e9
    clocks = clk.summary()
    # the distribution of single steps (a separate run of the same steps, an event at each step
    # boundary)
    nper = max(1, min(args.steps, 40))
    L.p3dfft_gb300_synchronize()
    L.p3dfft_gb300_event_record(10)
    for i in range(nper):
        step(d_in.ptr, d_out.ptr)
        L.p3dfft_gb300_event_record(11 + i)
    per_step = sorted(L.p3dfft_gb300_event_elapsed_ms(10 + i, 11 + i) for i in range(nper))
    step_dist = {"steps": nper, "median_ms": float(np.median(per_step)),
                 "p10_ms": float(np.percentile(per_step, 10)), "p90_ms": float(np.percentile(per_step, 90))}

    # ---- full-size properties: normalised round trip recovers the derivative field ----
    y = np.empty(p3d.storage_shape(GD, MO1), np.float64)
    d_out.download(y)

    # ---- per-stage profile (dominant kernel for the roofline) ----
    nst_f = len(f.stages())
    ms_f = (ctypes.c_double * 8)()
    ms_b = (ctypes.c_double * 8)()
    L.p3dfft_gb300_profile_stages(f.handle, ctypes.c_void_p(d_in.ptr), ctypes.c_void_p(d_spec.ptr), IDIR, 5, ms_f, 8)
    L.p3dfft_gb300_profile_stages(b.handle, ctypes.c_void_p(d_spec.ptr), ctypes.c_void_p(d_out.ptr), -1, 5, ms_b, 8)
    stages = []
    for plan, msv in ((f, ms_f), (b, ms_b)):
        pst = plan.stages(executed=True)
        for i, st in enumerate(pst):
            dt1 = 1 if st["type"] in (5,) else 2
            dt2 = 1 if st["type"] in (7,) else 2
            bytes_ = 8 * (dt1 * int(np.prod(st["gdims1"])) + dt2 * int(np.prod(st["gdims2"])))
            # complex FFT points of the stage (an even-length R2C / C2R runs a half-length FFT)
            pts = int(np.prod(st["gdims1"] if dt2 == 2 else st["gdims2"])) // (2 if st["type"] in (5, 7) else 1)
            stages.append({"dim": st["dim"], "type": st["type"], "ms": msv[i], "bytes": bytes_,
                           "points": pts, "kernel": kernel_id(st, arith, GD, ff_variant(pst, i, arith))})
    # dominant kernel = the instantiation with the largest total time per step
    per_kernel = {}
    for s in stages:
        agg = per_kernel.setdefault(s["kernel"], {"ms": 0.0, "bytes": 0, "points": 0, "launches": 0})
        agg["ms"] += s["ms"]
        agg["bytes"] += s["bytes"]
        agg["points"] += s["points"]
        agg["launches"] += 1
    kernel_key = max(per_kernel, key=lambda k: per_kernel[k]["ms"])
    dk = per_kernel[kernel_key]
    peak, peak_kind = measured_peak()
    achieved = dk["bytes"] / (dk["ms"] * 1e-3) / 1e9
    traffic = load_traffic(kernel_key) if GD == (512, 512, 512) else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": kernel_key, "peak_source": peak_kind,
                "launches_per_step": dk["launches"], "bytes_per_launch": dk["bytes"] // dk["launches"],
                "ms_per_launch": dk["ms"] / dk["launches"], "step_share": dk["ms"] / sum(s["ms"] for s in stages),
                "whole_step_frac": value / world / peak,
                # compulsory traffic (each real field and each spectrum once: 2*S_r + 2*S_c) over
                # the step time, against the peak
                "compulsory_bytes_per_step": 2 * S_R + 2 * S_C,
                "compulsory_frac": (2 * S_R + 2 * S_C) / (ms_step * 1e-3) / 1e9 / peak,
                "stages_ms": [round(s["ms"], 4) for s in stages]}
    # float-float kernels are compute-side bound: instruction issue (warp instructions per launch,
    # ncu count per point x the launch's points, over the live duration, against 4 per SM per
    # clock) and the FMA pipe (FP32 operations against 128 per SM per clock), both at the median
    # SM clock sampled during the timed region
    n_sm = L.p3dfft_gb300_sm_count()
    ipp = load_instr(kernel_key) if arith else None
    fpp = load_instr(kernel_key, "FP32OPS") if arith else None
    if n_sm and clocks.get("sm_mhz"):
        clk = clocks["sm_mhz"] * 1e6
        per_s = dk["points"] / dk["launches"] / (roofline["ms_per_launch"] * 1e-3)
        if ipp:
            ach, pk = ipp * per_s, 4.0 * n_sm * clk
            roofline["issue"] = {"bound": "instruction issue", "achieved": ach, "peak": pk, "unit": "warp-inst/s",
                                 "frac": ach / pk, "warp_inst_per_point": ipp, "sms": n_sm, "sm_mhz": clocks["sm_mhz"]}
        if fpp:
            ach, pk = fpp * per_s, 128.0 * n_sm * clk
            roofline["fp32_pipe"] = {"bound": "FMA pipe (FP32 operations)", "achieved": ach, "peak": pk,
                                     "unit": "FP32 op/s", "frac": ach / pk, "fp32_ops_per_point": fpp}
            # the HBM fraction this kernel could reach with its FMA pipe 100% busy: the time its
            # FP32 operations take at the pipe's peak against the time its bytes take at the
            # HBM peak
            t_ops = fpp * dk["points"] / dk["launches"] / pk
            t_hbm = dk["bytes"] / dk["launches"] / (peak * 1e9)
            roofline["compute_ceiling_frac"] = min(1.0, t_hbm / t_ops)
    # the dominant kernel's per-point counts and DRAM traffic come from the committed ncu
    # summaries under profiles/ (one small-case capture each), not from this run
    roofline["counts_source"] = "profiles/ (committed ncu summaries: TRAFFIC, INSTR, FP32OPS lines)"
    if n_sm and clocks.get("sm_mhz"):
        # the step's FFT flops (2.5 V log2 V per direction) against the native FP64 pipe's peak
        # (DFMA at the 1.75 thread instructions per SM per clock measured on this part, 2 flops
        # each): what the float-float arithmetic delivers beyond that pipe
        fl = 2 * 2.5 * GD[0] * GD[1] * GD[2] * np.log2(float(GD[0] * GD[1] * GD[2]))
        pk = 2 * 1.75 * n_sm * clocks["sm_mhz"] * 1e6
        roofline["fp64_pipe_equivalent"] = {"flops_per_step": fl, "achieved_tflops": fl / (ms_step * 1e-3) / 1e12,
                                            "native_fp64_peak_tflops": pk / 1e12,
                                            "ratio_to_native_peak": fl / (ms_step * 1e-3) / pk}

    # ---- e2e: pinned host buffers through the public API ----
    hin = p3d.PinnedArray(p3d.storage_shape(GD, MO1), np.float64)
    hout = p3d.PinnedArray(p3d.storage_shape(GD, MO1), np.float64)
    hin.array[...] = x
    n_e2e = max(3, min(args.steps, 20))

    def e2e_run(pin=None, pout=None):
        pin, pout = pin or hin.ptr, pout or hout.ptr
        for _ in range(2):
            step(pin, pout)
        L.p3dfft_gb300_synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            step(pin, pout)  # host in (exec_deriv) and host out (exec), each call synchronous
        L.p3dfft_gb300_synchronize()
        return max_over_ranks((time.perf_counter() - t0) / n_e2e * 1e3)

    # page-locked host arrays: the x stages read / write them over NVLink-C2C (default), or
    # staged through HBM with copies
    modes_ms = {}
    for mode, key in ((False, "staged_both"), ("in", "direct_in_staged_out"), ("out", "staged_in_direct_out"),
                      (True, "direct_both")):
        p3d.set_host_direct(mode)
        modes_ms[key] = e2e_run()
    p3d.set_host_direct(True)
    # A/B: staged copies with the first / last two stages pipelined behind them (default) or
    # the first / last stage alone
    p3d.set_host_direct(False)
    p3d.set_host_pipeline(False)
    modes_ms["staged_both_not_pipelined"] = e2e_run()
    p3d.set_host_pipeline(True)
    p3d.set_host_direct(True)
    # A/B: direct host access with the x stages on capped grids of persistent CTAs and the y
    # stages beside them slab by slab (default), or stage after stage
    p3d.set_link_ctas(0)
    modes_ms["direct_both_not_pipelined"] = e2e_run()
    p3d.set_link_ctas(-1)
    # pageable host arrays (plain numpy memory, pages already touched): staged through HBM by the
    # copies (default), or read / written in place through the host's page tables
    x_pg, y_pg = np.array(x), np.zeros_like(x)
    modes_ms["pageable_staged"] = e2e_run(x_pg.ctypes.data, y_pg.ctypes.data)
    p3d.set_pageable_direct(True)
    if p3d.get_pageable_direct() == 1:
        modes_ms["pageable_direct"] = e2e_run(x_pg.ctypes.data, y_pg.ctypes.data)
    p3d.set_pageable_direct(False)
    del x_pg, y_pg
    e2e_staged_ms = modes_ms["staged_both"]
    e2e_ms = modes_ms["direct_both"]
    e2e = {"value": ALG_BYTES * world / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s", "h2d_bytes_per_step": S_R,
           "d2h_bytes_per_step": S_R, "ms_per_step": e2e_ms,
           "host_io": "page-locked host arrays read by the x R2C stage and written by the x C2R stage over "
                      "NVLink-C2C, each on a capped grid of persistent CTAs with the y stage beside it slab by slab",
           "staged_copies": {"ms_per_step": e2e_staged_ms,
                             "value": ALG_BYTES * world / (e2e_staged_ms * 1e-3) / 1e9},
           "host_io_modes_ms": modes_ms,
           "link_stage_ctas": "1 per SM (FP64)"}
    rt_err = float(np.linalg.norm(hout.array - y) / max(np.linalg.norm(y), 1e-300))
    # per-phase breakdown of the end-to-end step run stage after stage (CUDA events around each
    # stage, page-locked host arrays read / written directly by the x stages): the host-link-bound
    # x R2C and x C2R, the on-device stages between them, and the host time outside the stages
    # (against the stage-after-stage step; the default step overlaps the y stages with the x)
    ph_f, ph_b = (ctypes.c_double * 8)(), (ctypes.c_double * 8)()
    nf = L.p3dfft_gb300_profile_stages(f.handle, ctypes.c_void_p(hin.ptr), ctypes.c_void_p(d_spec.ptr), IDIR, 3, ph_f, 8)
    nb = L.p3dfft_gb300_profile_stages(b.handle, ctypes.c_void_p(d_spec.ptr), ctypes.c_void_p(hout.ptr), -1, 3, ph_b, 8)
    if nf > 0 and nb > 0:
        fwd_ms, bwd_ms = list(ph_f)[:nf], list(ph_b)[:nb]
        link_ms = fwd_ms[0] + bwd_ms[-1]
        dev_ms = sum(fwd_ms[1:]) + sum(bwd_ms[:-1])
        e2e["phases_ms"] = {
            "x_r2c_reading_host": fwd_ms[0], "on_device_stages": dev_ms, "x_c2r_writing_host": bwd_ms[-1],
            "outside_stage_kernels": modes_ms["direct_both_not_pipelined"] - link_ms - dev_ms,
            "overlapped_by_link_pipelining": modes_ms["direct_both_not_pipelined"] - e2e_ms,
            # the pipelined schedule's floor: the link-bound x stages, the z stages (they need the
            # whole field) and the thin y slab (1/16 of the planes) in each direction outside the
            # link time
            "pipelined_schedule_floor": link_ms + fwd_ms[2] + bwd_ms[0] + (fwd_ms[1] + bwd_ms[1]) / max(
                2, int(os.environ.get("P3DFFT_GB300_LINK_TAIL", "16"))),
            "forward_stages": fwd_ms, "backward_stages": bwd_ms,
            "host_link_GBps": {"h2d_in_x_r2c": S_R / (fwd_ms[0] * 1e-3) / 1e9,
                               "d2h_in_x_c2r": S_R / (bwd_ms[-1] * 1e-3) / 1e9}}
    del hin, hout

    # ---- full-size parity: the 512^3 forward with fused d/dz against the reference's own output ----
    parity = full_size_parity(p3d, f, b, d_in, d_spec, d_out)
    d_in.upload(x)

    # ---- the other FP64 arithmetic and the FP32 form, same workload, device-resident ----
    def timed(fh, bh, din, dspec, dout, steps):
        for _ in range(3):
            p3d.check(L.p3dfft_gb300_exec3d(fh, ctypes.c_void_p(din), ctypes.c_void_p(dspec), IDIR, 0))
            p3d.check(L.p3dfft_gb300_exec3d(bh, ctypes.c_void_p(dspec), ctypes.c_void_p(dout), -1, 0))
        L.p3dfft_gb300_synchronize()
        L.p3dfft_gb300_event_record(2)
        for _ in range(steps):
            p3d.check(L.p3dfft_gb300_exec3d(fh, ctypes.c_void_p(din), ctypes.c_void_p(dspec), IDIR, 0))
            p3d.check(L.p3dfft_gb300_exec3d(bh, ctypes.c_void_p(dspec), ctypes.c_void_p(dout), -1, 0))
        L.p3dfft_gb300_event_record(3)
        return L.p3dfft_gb300_event_elapsed_ms(2, 3) / steps

    forms = {}
    if arith:
        # the same float-float round trip with IEEE-double intermediate fields (A/B of the
        # float-float intermediates)
        p3d.set_ff_intermediates(False)
        ms_ieee = timed(f.handle, b.handle, d_in.ptr, d_spec.ptr, d_out.ptr, max(5, args.steps // 5))
        y_ieee = d_out.download(np.empty_like(y))
        mf, mb = (ctypes.c_double * 8)(), (ctypes.c_double * 8)()
        nf = L.p3dfft_gb300_profile_stages(f.handle, ctypes.c_void_p(d_in.ptr), ctypes.c_void_p(d_spec.ptr), IDIR, 5, mf, 8)
        nb = L.p3dfft_gb300_profile_stages(b.handle, ctypes.c_void_p(d_spec.ptr), ctypes.c_void_p(d_out.ptr), -1, 5, mb, 8)
        p3d.set_ff_intermediates(True)
        forms["fp64_float_float_ieee_intermediates"] = {
            "ms_per_step": ms_ieee, "value": ALG_BYTES / (ms_ieee * 1e-3) / 1e9, "unit": "GB/s",
            "rel_l2_vs_headline": float(np.linalg.norm(y_ieee - y) / np.linalg.norm(y)),
            "stages_ms": [round(v, 4) for v in list(mf)[:max(nf, 0)] + list(mb)[:max(nb, 0)]]}
    p3d.set_fp64_arith(1 - arith)
    ms_other = timed(f.handle, b.handle, d_in.ptr, d_spec.ptr, d_out.ptr, max(3, args.steps // 10))
    y_other = d_out.download(np.empty_like(y))
    p3d.set_fp64_arith(arith)
    forms["fp64_native" if arith else "fp64_float_float"] = {
        "ms_per_step": ms_other, "value": ALG_BYTES / (ms_other * 1e-3) / 1e9, "unit": "GB/s",
        "rel_l2_vs_headline": float(np.linalg.norm(y_other - y) / np.linalg.norm(y))}
    if arith and n_sm and clocks.get("sm_mhz"):
        # native FP64 against the FP64 pipe: the usual 2.5 V log2 V flops per direction, against
        # DFMA at the 1.75 thread instructions per SM per clock measured on this part (2 flops each)
        fl = 2 * 2.5 * GD[0] * GD[1] * GD[2] * np.log2(float(GD[0] * GD[1] * GD[2]))
        pk = 2 * 1.75 * n_sm * clocks["sm_mhz"] * 1e6
        forms["fp64_native"]["fp64_pipe"] = {"flops_per_step": fl, "achieved_tflops": fl / (ms_other * 1e-3) / 1e12,
                                             "peak_tflops": pk / 1e12, "frac": fl / (ms_other * 1e-3) / pk,
                                             "hbm_frac": ALG_BYTES / (ms_other * 1e-3) / 1e9 / peak}
    f32 = p3d.Transform3D((4, 8, 8), GD, MO1, GD2, MO2, -1, 0)
    b32 = p3d.Transform3D((6, 10, 10), GD2, MO2, GD, MO1, 0, -1)
    d_in32, d_spec32, d_out32 = p3d.DeviceArray(S_R // 2), p3d.DeviceArray(S_C // 2), p3d.DeviceArray(S_R // 2)
    d_in32.upload(x.astype(np.float32))
    ms32 = timed(f32.handle, b32.handle, d_in32.ptr, d_spec32.ptr, d_out32.ptr, args.steps)
    y32 = d_out32.download(np.empty(y.shape, np.float32)).astype(np.float64)
    forms["fp32"] = {"ms_per_step": ms32, "value": (ALG_BYTES // 2) / (ms32 * 1e-3) / 1e9, "unit": "GB/s",
                     "round_trips_per_s": 1e3 / ms32, "speedup_vs_fp64_transforms_per_s": ms_step / ms32,
                     "rel_l2_vs_fp64": float(np.linalg.norm(y32 - y) / np.linalg.norm(y)),
                     "twiddles": "split (compensated) products on the 512-point lines, FP64-generated tables"}
    # A/B: plain FP32 twiddles on the long lines too
    p3d.set_fp32_split_twiddles(False)
    ms32p = timed(f32.handle, b32.handle, d_in32.ptr, d_spec32.ptr, d_out32.ptr, args.steps)
    y32p = d_out32.download(np.empty(y.shape, np.float32)).astype(np.float64)
    p3d.set_fp32_split_twiddles(True)
    forms["fp32"]["plain_twiddles"] = {"ms_per_step": ms32p,
                                       "rel_l2_vs_fp64": float(np.linalg.norm(y32p - y) / np.linalg.norm(y))}
    forms["fp32"]["line_error_vs_fp64_by_length"] = fp32_line_errors(p3d)

    # A/B: TMA-staged tile loads (the default) against per-thread global loads, in the FP32 stages
    # whose lines are contiguous (per-stage CUDA-event times both ways)
    def fp32_stage_ms():
        mf, mb = (ctypes.c_double * 8)(), (ctypes.c_double * 8)()
        nf = L.p3dfft_gb300_profile_stages(f32.handle, ctypes.c_void_p(d_in32.ptr), ctypes.c_void_p(d_spec32.ptr), IDIR, 5, mf, 8)
        nb = L.p3dfft_gb300_profile_stages(b32.handle, ctypes.c_void_p(d_spec32.ptr), ctypes.c_void_p(d_out32.ptr), -1, 5, mb, 8)
        return [round(v, 4) for v in list(mf)[:max(nf, 0)] + list(mb)[:max(nb, 0)]]

    c0 = p3d.tma_launch_count()
    p3d.check(L.p3dfft_gb300_exec3d(f32.handle, ctypes.c_void_p(d_in32.ptr), ctypes.c_void_p(d_spec32.ptr), IDIR, 0))
    p3d.check(L.p3dfft_gb300_exec3d(b32.handle, ctypes.c_void_p(d_spec32.ptr), ctypes.c_void_p(d_out32.ptr), -1, 0))
    L.p3dfft_gb300_synchronize()
    tma_stages = p3d.tma_launch_count() - c0
    y32_t = d_out32.download(np.empty(y.shape, np.float32))
    st_tma = fp32_stage_ms()
    p3d.set_fp32_tma(False)
    ms32n = timed(f32.handle, b32.handle, d_in32.ptr, d_spec32.ptr, d_out32.ptr, args.steps)
    y32_n = d_out32.download(np.empty(y.shape, np.float32))
    st_lsu = fp32_stage_ms()
    p3d.set_fp32_tma(True)
    forms["fp32"]["tma"] = {"stages_per_round_trip": tma_stages, "ms_per_step_per_thread_loads": ms32n,
                            "bit_identical_to_per_thread_loads": bool(np.array_equal(y32_t, y32_n)),
                            "stages_ms_tma": st_tma, "stages_ms_per_thread_loads": st_lsu,
                            "status_word": p3d.device_status()}
    del d_in32, d_spec32, d_out32, f32, b32
    forms["mixed_types_384x256x257"] = mixed_types_workload(p3d, L, max(5, args.steps // 5), arith)
    if not args.no_batch:
        del d_in, d_spec, d_out  # free HBM for the batch buffers
        forms["batched_uneven"] = batch_workload(p3d, L, max(3, min(args.steps, 10)), 3)
    if not args.no_serve:
        forms["serving"] = serve_workload(p3d, n_jobs=args.serve_jobs, nslots=args.serve_slots)

    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(world),
            "fp64_arith": "float-float (FP32 pipe, ~48-bit)" if arith else "native FP64 (DFMA)",
            "roofline": roofline, "e2e": e2e, "clocks": clocks, "gpu_launches": launches,
            "step_distribution": step_dist,
            "host_vs_device_rel_diff": rt_err, "parity": parity, "other_forms": forms}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample()
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()


if __name__ == "__main__":
    main()
