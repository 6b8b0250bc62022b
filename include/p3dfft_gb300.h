/*
 * GB300 extensions of the P3DFFT++ C interface (libp3dfft_gb300.so).
 *
 * The reference's C++ templates (transform3D<T1,T2>, transplan<T1,T2>) are header-only
 * wrappers over these plain-C entry points, so every exported symbol takes only ints and
 * pointers.  None of these has a counterpart in the reference's C wrappers unless stated.
 */
#ifndef P3DFFT_GB300_EXT_H
#define P3DFFT_GB300_EXT_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error side channel (the reference reports errors with printf / MPI_Abort) ---- */
#define P3DFFT_OK 0
#define P3DFFT_ERR_BAD_ARG 1
#define P3DFFT_ERR_UNSUPPORTED 2
#define P3DFFT_ERR_CUDA 3
#define P3DFFT_ERR_NO_DEVICE 4
#define P3DFFT_ERR_TOO_LARGE 5
#define P3DFFT_ERR_PLAN 6
#define P3DFFT_ERR_ALIGN 7
/* last error code of this thread's calls into the library, cleared by p3dfft_clear_error */
int p3dfft_last_error(void);
const char *p3dfft_last_error_string(void);
void p3dfft_clear_error(void);

/* ---- execution controls ---- */
/* CUDA stream used by every launch (default 0, the legacy default stream) */
void p3dfft_gb300_set_stream(void *cuda_stream);
/* 1 (default): exec returns after the result is in `out`; 0: device-pointer execs return
 * once the work is queued on the stream (host-pointer execs always synchronise). */
void p3dfft_gb300_set_sync(int sync);
/* 1 (default): page-locked host arrays (cudaHostAlloc, cudaHostRegister,
 * p3dfft_gb300_host_alloc_pinned) are read by the first stage and written by the last stage
 * directly over NVLink-C2C, without staging copies; 2: inputs only; 3: outputs only; 0: always
 * stage host arrays through HBM (slab by slab, the copies overlapped with the stage, for fields
 * of 32 MB and more).  Pageable host arrays are always staged.  P3DFFT_GB300_HOST_DIRECT=0 /
 * in / out sets 0 / 2 / 3 at start-up. */
void p3dfft_gb300_set_host_direct(int on);
/* 1 (default): when host arrays are staged through HBM (pageable arrays, or host_direct 0), the
 * first two stages run slab by slab behind the per-slab host-to-device copies (slabs along the dim
 * neither transforms; the second stage on a second stream), and the last two stages likewise
 * ahead of the per-slab copies back (fields of 32 MB and more, plans of 3+ stages, the slab dim
 * the slowest of the staged layout).  0: the first / last stage alone overlaps its copies.
 * P3DFFT_GB300_PIPELINE=0 sets 0 at start-up. */
void p3dfft_gb300_set_host_pipeline(int on);
int p3dfft_gb300_get_host_pipeline(void);
/* n > 0: a first stage that reads a page-locked host array directly (or a last stage that writes
 * one) runs with at most n CTAs, each walking its tiles, slab by slab, while the next (previous)
 * stage runs on the SMs it leaves free, one slab behind (fields of 32 MB and more, plans of 3+
 * stages, host pipelining on, R2C first / C2R last stages of FFT length 64..2048).  0: those
 * stages run alone, stage after stage.  n < 0: the default, P3DFFT_GB300_LINK_CTAS when set,
 * else one CTA per SM for FP64 stages and two per SM for FP32.  get returns the cap set (or the
 * variable's), -1 for the default. */
void p3dfft_gb300_set_link_ctas(int n);
int p3dfft_gb300_get_link_ctas(void);
/* 1: pageable host arrays (plain malloc / new) are read and written by the first / last stage in
 * place, like page-locked ones, where the device accesses pageable memory through the host's
 * page tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables, e.g. Grace with NVLink-C2C);
 * elsewhere, and with 0 (the default), pageable arrays are staged through HBM.
 * P3DFFT_GB300_PAGEABLE_DIRECT=1 sets 1 at start-up.  get: 1 on, 0 off, -1 not supported by the
 * device. */
void p3dfft_gb300_set_pageable_direct(int on);
int p3dfft_gb300_get_pageable_direct(void);
/* Arithmetic of FP64 stages: 1 = float-float on the FP32 pipe (default; ~48-bit significand,
 * ~1e-14 relative L2 per 3D transform), 0 = native FP64 DFMA (slow on GB300).  The initial value
 * can be set with P3DFFT_GB300_FP64_ARITH=native. */
void p3dfft_gb300_set_fp64_arith(int mode);
int p3dfft_gb300_get_fp64_arith(void);
/* 1 (default): reproduce two reference behaviours whose results are deterministic, so outputs
 * equal the reference's: compute_deriv differentiates along storage axis imo[idir], the logical
 * dim whose storage rank is idir (reference build/deriv.C:89-93; differs from the storage axis of
 * dim idir only for the 3-cycle memory orders), and a 1D plan whose input and output orders both
 * have the transform dim non-leading reads its input as stored in order swap0(mo1, dim) (reference
 * build/templ.C:1015-1023, where find_m overwrites the plan's input order).  0: differentiate
 * along logical dim idir and read 1D inputs in their declared order.  The initial value can be
 * set with P3DFFT_GB300_REFERENCE_COMPAT=0. */
void p3dfft_gb300_set_reference_compat(int on);
int p3dfft_gb300_get_reference_compat(void);
/* 1 (default): with float-float FP64 arithmetic, consecutive stages that both run the specialised
 * float-float kernels pass their intermediate field as packed float-float pairs at per-line
 * power-of-two scales (plus a side array of the scales) instead of IEEE doubles, which saves the
 * conversions; the caller's input and output are IEEE doubles either way.  0: every stage reads
 * and writes IEEE doubles.  The initial value can be set with P3DFFT_GB300_FF_INTERMEDIATE=0. */
void p3dfft_gb300_set_ff_intermediates(int on);
int p3dfft_gb300_get_ff_intermediates(void);
/* 1 (default): FP32 stages whose FFT length is 512, 1024 or 2048 multiply by split twiddles, each
 * the FP32 pair (hi, lo) of its long-double value, as a * hi + a * lo (compensated twiddle
 * products: the twiddle adds no rounding of its own); 0: FP32 twiddles, most formed as products
 * of two table entries.  The initial value can be set with P3DFFT_GB300_FP32_SPLIT_TWIDDLES=0. */
void p3dfft_gb300_set_fp32_split_twiddles(int on);
int p3dfft_gb300_get_fp32_split_twiddles(void);
/* 1 (default): FP32 C2C / R2C stages in device memory fetch each tile by TMA (a tensor map over
 * the input, cp.async.bulk.tensor into shared memory) instead of per-thread global loads, where
 * the tile is a box: lines contiguous and evenly spaced, or (C2C) the tile dim contiguous and a
 * multiple of the tile's lines; even lengths 2^a*3^b*5^c from 32 whose first radix equals the
 * points per thread.  0: always per-thread loads.  The initial value can be set with
 * P3DFFT_GB300_FP32_TMA=0. */
void p3dfft_gb300_set_fp32_tma(int on);
int p3dfft_gb300_get_fp32_tma(void);
/* The device status word: nonzero after a kernel's bounded wait ran out (the tile was skipped,
 * the output is invalid).  clear != 0 resets it.  Synchronous. */
int p3dfft_gb300_device_status(int clear);
/* Test hook: the next TMA-staged launch waits for 16 bytes its copies never deliver, so every
 * tile's wait runs out after 20 ms and sets the status word (no tile is transformed). */
void p3dfft_gb300_inject_tma_stall(void);
/* TMA-staged stage launches since the library was loaded */
long long p3dfft_gb300_tma_launch_count(void);

/* ---- planning / execution by explicit grid descriptions (1x1x1 processor grid) ----
 * A grid is (gdims[3], mem_order[3], dim_conj_sym).  Returns a handle >= 0, or -1 with the
 * error recorded.  Type IDs are the reference's (0..43, p3dfft::setup order). */
int p3dfft_gb300_plan3d(const int types[3], const int gdims1[3], const int mo1[3], int dcs1,
                        const int gdims2[3], const int mo2[3], int dcs2);
/* idir < 0: plain transform; 0..2: fused spectral derivative along that logical dim. */
int p3dfft_gb300_exec3d(int plan, const void *in, void *out, int idir, int OW);
int p3dfft_gb300_destroy3d(int plan);
/* dt1 / dt2 (1 real, 2 complex) and precision (4/8) of a 3D plan */
int p3dfft_gb300_plan3d_types(int plan, int *dt1, int *dt2, int *prec);
/* Stage list of a 3D plan: per stage 1+1+3+3+1+3+3+1 = 16 ints
 * (type, dim, gdims1[3], mo1[3], dcs1, gdims2[3], mo2[3], dcs2).  Returns the stage count. */
int p3dfft_gb300_plan3d_stages(int plan, int *info, int max_stages);
/* The schedule the executor runs, same format.  It applies the same 1D transform to each dim as
 * the stage list above, between the same input and output grids, but may order the dims
 * differently (R2C stays first, C2R last) and choose other intermediate memory orders so that
 * every stage reads and writes long contiguous runs; P3DFFT_GB300_REFERENCE_SCHEDULE=1 runs the
 * reference's stage list instead. */
int p3dfft_gb300_plan3d_exec_stages(int plan, int *info, int max_stages);

int p3dfft_gb300_plan1d(int type, const int gdims1[3], const int mo1[3], int dcs1,
                        const int gdims2[3], const int mo2[3], int dcs2, int dim);
int p3dfft_gb300_exec1d(int plan, const void *in, void *out, int OW);
int p3dfft_gb300_destroy1d(int plan);

/* compute_deriv on a complex field of grid (gdims, mo, dcs); prec 4 or 8, idir 0-based */
int p3dfft_gb300_compute_deriv(int prec, const void *in, void *out, const int gdims[3],
                               const int mo[3], int dcs, int idir);

/* ---- autotuner (no counterpart in the reference) ----
 * For every stage of a plan, times each kernel choice the stage admits (engine: 1 specialised
 * kernel with a compile-time radix plan and tile shape, 2 register engine, 3 generic mixed-radix
 * engine; talt: the tile's consecutive lines along the first (0) or second (1) batch dim) and keeps
 * the fastest.  Choices are cached per stage (kind, precision, FP64 arithmetic, dims, strides), so
 * plans that share a stage share its tuning.  is1d selects a 1D plan handle.  With set_autotune(1)
 * every plan is tuned at its first exec.  The cache can be saved and loaded as a text file. */
void p3dfft_gb300_set_autotune(int on);
int p3dfft_gb300_autotune(int plan, int is1d);
/* per stage: engine (0 = heuristic), talt, measured ms; returns the stage count */
int p3dfft_gb300_plan_tuning(int plan, int is1d, int *engine, int *talt, double *ms, int max_stages);
/* forces a stage's kernel choice (engine 0 = heuristic) */
int p3dfft_gb300_plan_set_engine(int plan, int is1d, int stage, int engine, int talt);
int p3dfft_gb300_tune_cache_save(const char *path);
int p3dfft_gb300_tune_cache_load(const char *path);
void p3dfft_gb300_tune_cache_clear(void);

/* ---- allocation-free execution (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc (an application that gives all device memory to its own
 * allocator at start-up, a real-time loop that may not take cudaMalloc's implicit device
 * synchronisation, a plugin host that forbids device allocations): runs a 3D plan like
 * p3dfft_gb300_exec3d, with
 * the intermediate fields and twiddle tables in a static device array of
 * P3DFFT_GB300_NOALLOC_BYTES that every GPU loading the library holds until exit.  `in` and
 * `out` must be device memory; each intermediate field must fit in
 * p3dfft_gb300_noalloc_max_field_bytes() (about 95 MiB, e.g. a 128^3 or 256x256x128 FP64
 * R2C round trip), larger transforms are rejected with P3DFFT_ERR_TOO_LARGE.  The first call on
 * a device resolves the array's device address (cudaGetSymbolAddress) and should come before
 * any stream capture.  Each call stages the plan's twiddle tables through a static host array
 * that the next call overwrites, so a call made while the library stream is being captured is
 * refused with P3DFFT_ERR_UNSUPPORTED.  Calls share the arrays: calls that overlap on the GPU
 * race.  Stages whose tuned engine needs the library's cached tables run the heuristic engine. */
#define P3DFFT_GB300_NOALLOC_BYTES (192ull << 20)
int p3dfft_gb300_exec3d_noalloc(int plan, const void *in, void *out, int idir);
long long p3dfft_gb300_noalloc_max_field_bytes(void);

/* ---- batched execution of independent transforms (no counterpart in the reference) ----
 * A batch holds jobs; a job is an ordered list of steps (3D plan, device in, device out, idir), e.g. an
 * R2C forward then its C2R backward.  Jobs are independent: by default they run as grouped
 * launches (see batch_set_grouped), else on `nbranches` concurrent streams (0 = 8), each with its
 * own scratch fields.  The first batch_exec runs the
 * jobs and records them into one CUDA graph; later execs replay the graph with one launch on the
 * library stream.  Pointers are captured: keep the buffers allocated while the batch exists.
 * batch_add after an exec, a change of FP64 arithmetic or batch_set_graph re-records the graph. */
int p3dfft_gb300_batch_create(int nbranches);
int p3dfft_gb300_batch_add(int batch, int job, int plan, const void *in, void *out, int idir);
int p3dfft_gb300_batch_set_graph(int batch, int on);
/* 1 (default): jobs with the same steps form a cohort; each stage of a cohort is one launch of its
 * specialised kernel over all the cohort's jobs' tiles; cohorts run on `nbranches` concurrent
 * streams.  2: work lists: the k-th stages of all jobs form level k, and within a level every
 * stage that runs the same specialised kernel (arithmetic, kind, FFT length) joins one launch
 * over all their tiles, whatever their grids, memory orders and buffers (a device list of
 * (stage, tile) items with each stage's parameters).  The launches go round-robin to the
 * `nbranches` streams, each waiting only for the launches that ran the previous stage of its own
 * jobs.  Set P3DFFT_GB300_LIST_PERSISTENT=1 before the first exec to cap each such launch's grid
 * at the resident CTAs (persistent CTAs walk the list).
 * 0: every job's stages launched separately, jobs spread over the streams. */
int p3dfft_gb300_batch_set_grouped(int batch, int on);
/* grouped launches one exec makes (0 in branch mode) */
int p3dfft_gb300_batch_groups(int batch);
int p3dfft_gb300_batch_exec(int batch);
/* kernels one batch_exec launches, and the field bytes its steps read and write */
long long p3dfft_gb300_batch_kernels(int batch);
double p3dfft_gb300_batch_field_bytes(int batch);
int p3dfft_gb300_batch_destroy(int batch);

/* ---- serving loop (no counterpart in the reference) ----
 * A server runs jobs (forward 3D plan, backward 3D plan, idir, in, out): `in` is copied into HBM,
 * transformed forward with the derivative along idir fused (idir < 0: none), transformed back,
 * and the result written to `out`.  in / out may be host memory (page-locked for overlap) or
 * device memory; the job's HBM fields come from the server's memory pool.  Jobs are admitted in
 * arrival order (bounded look-ahead) while a slot is free and their HBM need fits in the budget;
 * up to `nslots` jobs run concurrently on their own streams.  arrival_s >= 0 schedules the job's
 * arrival that many seconds after server creation (trace replay); < 0 means now. */
int p3dfft_gb300_server_create(long long hbm_budget_bytes, int nslots);
int p3dfft_gb300_server_submit(int srv, int plan_fwd, int plan_bwd, int idir, const void *in, void *out,
                               double arrival_s);
/* 0 done, 1 timeout (timeout_s < 0 waits indefinitely), < 0 failed with error -return */
int p3dfft_gb300_server_wait(int srv, int job, double timeout_s);
/* Failure injection on the host (for tests): the job's device allocation fails when it is
 * admitted, as if the memory pool had no room; the job then fails with P3DFFT_ERR_CUDA, its slot
 * and budget return to the server, and the other jobs are unaffected.  The job must still be
 * waiting for admission (submit it with a future arrival time). */
int p3dfft_gb300_server_inject_alloc_failure(int srv, int job);
int p3dfft_gb300_server_drain(int srv);
/* seconds since server creation */
double p3dfft_gb300_server_clock(int srv);
/* t[0] arrival, t[1] admission, t[2] completion, on the server clock */
int p3dfft_gb300_server_job_times(int srv, int job, double *t);
/* completed, failed, admitted, peak HBM bytes held by jobs, budget, most jobs running at once,
 * dispatcher seconds spent queueing jobs' work, and releasing their memory (up to n values) */
int p3dfft_gb300_server_stats(int srv, double *stats, int n);
int p3dfft_gb300_server_destroy(int srv);

/* ---- introspection and timers ---- */
/* loads every specialised stage kernel now instead of at its first launch (servers call this at
 * start-up so that no job pays a module load) */
int p3dfft_gb300_preload_kernels(void);
/* number of kernels this library launched since the last reset */
long long p3dfft_gb300_kernel_count(void);
void p3dfft_gb300_reset_kernel_count(void);
/* per-phase device time in seconds, accumulated when timing is enabled:
 * phase 0 trans_exec (no reorder), 1 reorder_trans (transform + layout change),
 * 2 reorder_out (pure reorder), 3 trans_deriv (stages with fused derivative),
 * 4 h2d, 5 d2h */
void p3dfft_gb300_enable_timers(int on);
double p3dfft_gb300_timer(int phase);
void p3dfft_gb300_reset_timers(void);
/* CUDA events on the library's stream (slots 0..63), for timing from a caller without its
 * own CUDA runtime; elapsed_ms synchronises on event b and returns -1 on error */
int p3dfft_gb300_event_record(int slot);
double p3dfft_gb300_event_elapsed_ms(int a, int b);
/* Runs a 3D plan `reps` times on device-resident buffers with an event between stages and
 * returns the stage count; ms[s] = average duration of stage s in milliseconds. */
int p3dfft_gb300_profile_stages(int plan, const void *in, void *out, int idir, int reps, double *ms,
                                int max_stages);
/* device-memory helpers for callers without a CUDA runtime of their own */
void *p3dfft_gb300_device_alloc(long long bytes);
void p3dfft_gb300_device_free(void *p);
/* page-locked host memory (fast staging for host-pointer execs) */
void *p3dfft_gb300_host_alloc_pinned(long long bytes);
void p3dfft_gb300_host_free_pinned(void *p);
int p3dfft_gb300_memcpy_h2d(void *dst, const void *src, long long bytes);
int p3dfft_gb300_memcpy_d2h(void *dst, const void *src, long long bytes);
int p3dfft_gb300_synchronize(void);
/* streaming multiprocessors of the library's device (0 when no device is usable) */
int p3dfft_gb300_sm_count(void);
/* library version string */
const char *p3dfft_gb300_version(void);

#ifdef __cplusplus
}
#endif
#endif
