// Internal interface between the host runtime (core.cpp) and the sm_103a kernels
// (stage_kernels.cu).  Not part of the public C ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include <vector>

namespace p3d {

// 1D transform kinds (the reference's trans_type1D flavours, build/init.C:121-731)
enum Kind { K_EMPTY = 0, K_R2C = 1, K_C2R = 2, K_C2C_FWD = 3, K_C2C_BWD = 4, K_R2R = 5 };
// FFTW r2r kinds
enum R2R { REDFT00 = 0, REDFT10, REDFT01, REDFT11, RODFT00, RODFT10, RODFT01, RODFT11 };

// Arithmetic used inside a stage for FP64 data: native DFMA, or float-float (two FP32 limbs,
// ~48-bit significand) on the FP32 pipe.  FP32 data always uses native FP32.
enum Arith { AR_NATIVE = 0, AR_DF = 1 };

// Error codes recorded by p3dfft_last_error()
enum Err {
  E_OK = 0,
  E_BAD_ARG = 1,
  E_UNSUPPORTED = 2,
  E_CUDA = 3,
  E_NO_DEVICE = 4,
  E_TOO_LARGE = 5,
  E_PLAN = 6,
  E_ALIGN = 7,
};

// One stage of a 3D (or 1D) plan, in logical-dimension terms: a 1D transform of `type kind`
// along logical dim L, reading a field of logical dims d1 stored with strides s1 (elements) and
// writing dims d2 with strides s2.  The two batch dims are the same size in and out.
struct StageDesc {
  int kind;       // Kind
  int r2r;        // R2R when kind == K_R2R
  int prec;       // 4 or 8
  int dt1, dt2;   // 1 real, 2 complex
  int L;          // transform dim
  int d1[3], d2[3];
  long long s1[3], s2[3];
  int deriv;      // fuse the i*k multiply (compute_deriv_loc)
  // tuning (0 = heuristic): engine 1 specialised kernel, 2 register engine, 3 generic engine
  // (radix passes only), 4 Bluestein engine;
  // talt 1 takes consecutive lines of a tile along the other batch dim
  int engine = 0;
  int talt = 0;
  // specialised kernels: at most this many CTAs, each walking the tiles with a grid stride
  // (0: one CTA per tile)
  int max_ctas = 0;
  int *tile_ctr = nullptr;  // with max_ctas: a zeroed counter for dynamic tile assignment
  // Float-float intermediate fields (float-float arithmetic, specialised C2C / R2C / C2R kernels
  // only; other launches with these set fail with E_UNSUPPORTED).  ffin: the input field holds
  // packed float-float values scaled per stored line; the scale of the value at logical
  // coordinates c is sin[sum_d c[d] * mi[d]].  ffout: store packed float-float values and each
  // line's scale at sout[sum_d c[d] * mo[d]] (mi / mo: 0 along the storing line's own dim).
  int ffin = 0, ffout = 0;
  const int *sin = nullptr;
  int *sout = nullptr;
  long long mi[3] = {0, 0, 0}, mo[3] = {0, 0, 0};
};
enum Engine { ENG_AUTO = 0, ENG_FAST = 1, ENG_FIXED = 2, ENG_GENERIC = 3, ENG_BLUESTEIN = 4 };

struct DeviceTables;  // twiddle-table cache, one per device

// Loads the module of every specialised stage kernel now (CUDA loads kernels lazily at their first
// launch, which would otherwise land inside the first transform of each length).
int preload_kernels();

// Twiddle tables a stage needs: W_tabN^k (and W_auxN^k for the generic DCT/DST kinds, auxN 0
// if none), in format fmt (0 double pairs, 1 float pairs, 2 float-float pairs).
struct TableNeed {
  int fmt, tabN, auxN;
  int aux_pass;  // 1: the aux table is the specialised kernels' per-pass twiddle rows of length auxN
  int ff = 0;    // the stage's kernel can read / write float-float intermediate fields
};
size_t table_bytes(int N, int fmt);
void fill_table(int N, int fmt, void *host_dst);
// Per-pass twiddle rows of the specialised kernels for FFT length N (fast_stage.cuh)
size_t pass_table_bytes(int N, int fmt);
void fill_pass_table(int N, int fmt, void *host_dst);
// Tables of the Bluestein engine for FFT length n
size_t blue_table_bytes(int n, int fmt);
void fill_blue_table(int n, int fmt, void *host_dst);

// Launch one stage on `stream`.  in != out is required (the host runtime guarantees it).
// Tables come from `tabs` (allocated on first use) unless `tw_given` is non-null, in which case
// tw_given / aux_given are used as they are.  With `tabs_out` non-null nothing is launched: the
// call only reports the tables the stage needs.
struct FastArgs;  // a specialised-kernel launch (fast_stage.cuh)
// With `fast_prep` non-null nothing is launched either: when the stage runs on a specialised
// kernel its launch is described in *fast_prep and E_OK returned, otherwise E_UNSUPPORTED.
int launch_stage(const StageDesc &d, const void *in, void *out, int arith, cudaStream_t stream,
                 DeviceTables *tabs, int *kernels_launched, const void *tw_given = nullptr,
                 const void *aux_given = nullptr, TableNeed *tabs_out = nullptr, FastArgs *fast_prep = nullptr);
// Whether the stage runs on a specialised kernel that honours StageDesc::max_ctas (nothing is
// launched; the stage's tables are loaded into `tabs`).
bool stage_cap_ok(const StageDesc &d, const void *in, void *out, int arith, DeviceTables *tabs);
// Device counters for capped launches (StageDesc::tile_ctr), kTileCounters of them, or nullptr.
constexpr int kTileCounters = 16;
int *tile_counters(DeviceTables *tabs);

// ---- grouped launches (batch runtime) ----
// One stage of one transform with its buffers, as the executor would launch it.
struct StageLaunch {
  StageDesc d;
  const void *src;
  void *dst;
  int arith;
};
// levels[k] holds the k-th stage of every transform of a set (e.g. a batch cohort).  A launch set
// runs level after level on one stream; within a level, stages that differ only in their buffers
// and run on a specialised kernel become one grouped launch over all their tiles, the others one
// launch each.  With work_list, stages that run the same specialised kernel (arithmetic, kind,
// length) become one grouped launch even when their grids, strides and tables differ.  A grouped
// launch is one k_fast_list launch over the members' (stage, tile) items, one CTA per item.
// Building uploads the groups' parameters and items.
struct LaunchSet;
LaunchSet *launch_set_build(const std::vector<std::vector<StageLaunch>> &levels, DeviceTables *tabs, int *err,
                            bool work_list = false);
int launch_set_run(LaunchSet *set, cudaStream_t stream, int *kernels_launched);
// the launches of level l, largest first (items 0 .. launch_set_items(set, l) - 1)
int launch_set_levels(const LaunchSet *set);
int launch_set_items(const LaunchSet *set, int level);
int launch_set_run_item(LaunchSet *set, int level, int item, cudaStream_t stream, int *kernels_launched);
// positions in levels[level] of the stages that item `item` runs
const std::vector<int> &launch_set_item_members(const LaunchSet *set, int level, int item);
int launch_set_groups(const LaunchSet *set);
void launch_set_destroy(LaunchSet *set);
// Pure permutation copy of an element size `esize` bytes field (EMPTY stages).
int launch_permute(const int d[3], const long long s1[3], const long long s2[3], int esize,
                   const void *in, void *out, cudaStream_t stream, int *kernels_launched);
// Standalone spectral derivative on a complex field (build/deriv.C:85-184), in may equal out.
// ref_axis: differentiate along storage axis imo[idir] as build/deriv.C:89-93 does (else along
// the storage axis of logical dim idir); the wavenumbers come from g in both cases
// FP32 specialised kernels on lines of 512, 1024 and 2048 points use split (compensated)
// twiddle products when on (the default)
bool fp32_split_twiddles();
void set_fp32_split_twiddles(bool on);
// FP32 C2C / R2C stages with contiguous, evenly spaced lines in device memory stage each tile's
// input by TMA (cp.async.bulk.tensor) when on (the default)
bool fp32_tma();
void set_fp32_tma(bool on);
// the next TMA launch's wait runs out (20 ms): the failure path of the bounded waits
void inject_tma_stall();
// TMA-staged launches so far
long long tma_launches();
// the device status word (nonzero: a kernel's bounded wait ran out and its tile was skipped);
// clear resets it.  Synchronous.
int device_status(DeviceTables *tabs, bool clear);
int launch_deriv(int prec, const int d[3], const long long s[3], int idir, int g, int ref_axis, const void *in,
                 void *out, cudaStream_t stream, int *kernels_launched);

DeviceTables *tables_create();
void tables_destroy(DeviceTables *);

// Smallest / largest supported transform length inside one CTA (per precision)
int max_line_len(int prec);

}  // namespace p3d
