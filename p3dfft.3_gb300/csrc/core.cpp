// Host runtime of the GB300 P3DFFT++ pipeline: type registry, grid model, 3D planner, stage
// executor, HBM buffer management and the C / Fortran / C++ entry points.
//
// Reference correspondence:
//   registry            p3dfft::setup            build/init.C:121-731
//   grid model          ProcGrid / DataGrid      build/init.C:1631-1863 (1x1x1 grid)
//   planner             transform3D ctor         build/templ.C:91-420, find_order 627-802,
//                                                swap0 816-858, excl 872-882, final_seq 422-435
//   1D plans            transplan::init_tr       build/templ.C:900-992
//   executor            transform3D::exec_deriv  build/exec.C:101-223 (stage loop)
//   C / Fortran ABI     build/wrap.C:85-796
// The executor keeps plans, twiddle tables and scratch fields resident in HBM (the reference
// allocates its temporaries on every call, exec.C:148-166) and runs one fused kernel per stage.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "p3dfft.h"

// ------------------------------------------------------------------------------------------
// Type-ID globals (values assigned by setup(), registration order of build/init.C:121-731)
extern "C" {
int P3DFFT_EMPTY_TYPE_SINGLE, P3DFFT_EMPTY_TYPE_DOUBLE, P3DFFT_EMPTY_TYPE_SINGLE_COMPLEX, P3DFFT_EMPTY_TYPE_DOUBLE_COMPLEX;
int P3DFFT_R2CFFT_S, P3DFFT_R2CFFT_D, P3DFFT_C2RFFT_S, P3DFFT_C2RFFT_D, P3DFFT_CFFT_FORWARD_S, P3DFFT_CFFT_FORWARD_D,
    P3DFFT_CFFT_BACKWARD_S, P3DFFT_CFFT_BACKWARD_D;
int P3DFFT_DCT1_REAL_S, P3DFFT_DCT1_REAL_D, P3DFFT_DST1_REAL_S, P3DFFT_DST1_REAL_D, P3DFFT_DCT1_COMPLEX_S,
    P3DFFT_DCT1_COMPLEX_D, P3DFFT_DST1_COMPLEX_S, P3DFFT_DST1_COMPLEX_D;
int P3DFFT_DCT2_REAL_S, P3DFFT_DCT2_REAL_D, P3DFFT_DST2_REAL_S, P3DFFT_DST2_REAL_D, P3DFFT_DCT2_COMPLEX_S,
    P3DFFT_DCT2_COMPLEX_D, P3DFFT_DST2_COMPLEX_S, P3DFFT_DST2_COMPLEX_D;
int P3DFFT_DCT3_REAL_S, P3DFFT_DCT3_REAL_D, P3DFFT_DST3_REAL_S, P3DFFT_DST3_REAL_D, P3DFFT_DCT3_COMPLEX_S,
    P3DFFT_DCT3_COMPLEX_D, P3DFFT_DST3_COMPLEX_S, P3DFFT_DST3_COMPLEX_D;
int P3DFFT_DCT4_REAL_S, P3DFFT_DCT4_REAL_D, P3DFFT_DST4_REAL_S, P3DFFT_DST4_REAL_D, P3DFFT_DCT4_COMPLEX_S,
    P3DFFT_DCT4_COMPLEX_D, P3DFFT_DST4_COMPLEX_S, P3DFFT_DST4_COMPLEX_D;
}

namespace p3dfft {
int EMPTY_TYPE_SINGLE, EMPTY_TYPE_DOUBLE, EMPTY_TYPE_SINGLE_COMPLEX, EMPTY_TYPE_DOUBLE_COMPLEX;
int R2CFFT_S, R2CFFT_D, C2RFFT_S, C2RFFT_D, CFFT_FORWARD_S, CFFT_FORWARD_D, CFFT_BACKWARD_S, CFFT_BACKWARD_D;
int DCT1_REAL_S, DCT1_REAL_D, DST1_REAL_S, DST1_REAL_D, DCT1_COMPLEX_S, DCT1_COMPLEX_D, DST1_COMPLEX_S, DST1_COMPLEX_D;
int DCT2_REAL_S, DCT2_REAL_D, DST2_REAL_S, DST2_REAL_D, DCT2_COMPLEX_S, DCT2_COMPLEX_D, DST2_COMPLEX_S, DST2_COMPLEX_D;
int DCT3_REAL_S, DCT3_REAL_D, DST3_REAL_S, DST3_REAL_D, DCT3_COMPLEX_S, DCT3_COMPLEX_D, DST3_COMPLEX_S, DST3_COMPLEX_D;
int DCT4_REAL_S, DCT4_REAL_D, DST4_REAL_S, DST4_REAL_D, DCT4_COMPLEX_S, DCT4_COMPLEX_D, DST4_COMPLEX_S, DST4_COMPLEX_D;
timer timers;
}  // namespace p3dfft

namespace p3d {

// ------------------------------------------------------------------------------------------
// error side channel
static thread_local int t_err = E_OK;
static thread_local char t_msg[512] = "no error";

static void set_err(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
static void set_err(int code, const char *fmt, ...) {
  t_err = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
  va_end(ap);
  if (getenv("P3DFFT_GB300_QUIET") == nullptr) fprintf(stderr, "P3DFFT++ (GB300) error: %s\n", t_msg);
}

// ------------------------------------------------------------------------------------------
// type registry
struct TypeInfo {
  int dt1, dt2, prec, kind, r2r;
  const char *name;
};
static TypeInfo g_types[44];
static bool g_setup_done = false;

static void build_registry() {
  // IDs 0..3: EMPTY single / double / single complex / double complex (init.C:132-179)
  const char *en[4] = {"Empty Type Single", "Empty Type Double", "Empty Type Single Complex", "Empty Type Double Complex"};
  for (int i = 0; i < 4; i++) g_types[i] = TypeInfo{i >= 2 ? 2 : 1, i >= 2 ? 2 : 1, (i & 1) ? 8 : 4, K_EMPTY, 0, en[i]};
  // 4..11: R2C S/D, C2R S/D, CFFT_FORWARD S/D, CFFT_BACKWARD S/D (init.C:216-311)
  g_types[4] = TypeInfo{1, 2, 4, K_R2C, 0, "Real-to-complex Fourier Transform, single precision"};
  g_types[5] = TypeInfo{1, 2, 8, K_R2C, 0, "Real-to-complex Fourier Transform double precision"};
  g_types[6] = TypeInfo{2, 1, 4, K_C2R, 0, "Complex-to-real Fourier Transform, single precision"};
  g_types[7] = TypeInfo{2, 1, 8, K_C2R, 0, "Complex-to-real Fourier Transform, double precision"};
  g_types[8] = TypeInfo{2, 2, 4, K_C2C_FWD, 0, "Complex-to-complex Fourier Transform, forward, single precision"};
  g_types[9] = TypeInfo{2, 2, 8, K_C2C_FWD, 0, "Complex-to-complex Fourier Transform, forward, double precision"};
  g_types[10] = TypeInfo{2, 2, 4, K_C2C_BWD, 0, "Complex-to-complex Fourier Transform, backward, single precision"};
  g_types[11] = TypeInfo{2, 2, 8, K_C2C_BWD, 0, "Complex-to-complex Fourier Transform, backward, double precision"};
  // 12..43: DCT1 DST1 DCT2 DST2 DCT3 DST3 DCT4 DST4 x {REAL_S, REAL_D, COMPLEX_S, COMPLEX_D}
  // (init.C:335-731).  The DCT4 IDs are registered with the DCT1 planners in the reference
  // (init.C:640, 652, 664, 676), so they compute REDFT00; that registration is kept.
  static const int fam_kind[8] = {REDFT00, RODFT00, REDFT10, RODFT10, REDFT01, RODFT01, REDFT00, RODFT11};
  static const char *fam_name[8] = {"DCT1", "DST1", "DCT2", "DST2", "DCT3", "DST3", "DCT4", "DST4"};
  for (int f = 0; f < 8; f++)
    for (int v = 0; v < 4; v++) {
      int id = 12 + 4 * f + v;
      int dt = v >= 2 ? 2 : 1;
      g_types[id] = TypeInfo{dt, dt, (v & 1) ? 8 : 4, K_R2R, fam_kind[f], fam_name[f]};
    }
}

static void assign_globals() {
  using namespace p3dfft;
  int *cpp[44] = {&EMPTY_TYPE_SINGLE, &EMPTY_TYPE_DOUBLE, &EMPTY_TYPE_SINGLE_COMPLEX, &EMPTY_TYPE_DOUBLE_COMPLEX,
                  &R2CFFT_S, &R2CFFT_D, &C2RFFT_S, &C2RFFT_D, &CFFT_FORWARD_S, &CFFT_FORWARD_D, &CFFT_BACKWARD_S,
                  &CFFT_BACKWARD_D, &DCT1_REAL_S, &DCT1_REAL_D, &DCT1_COMPLEX_S, &DCT1_COMPLEX_D, &DST1_REAL_S,
                  &DST1_REAL_D, &DST1_COMPLEX_S, &DST1_COMPLEX_D, &DCT2_REAL_S, &DCT2_REAL_D, &DCT2_COMPLEX_S,
                  &DCT2_COMPLEX_D, &DST2_REAL_S, &DST2_REAL_D, &DST2_COMPLEX_S, &DST2_COMPLEX_D, &DCT3_REAL_S,
                  &DCT3_REAL_D, &DCT3_COMPLEX_S, &DCT3_COMPLEX_D, &DST3_REAL_S, &DST3_REAL_D, &DST3_COMPLEX_S,
                  &DST3_COMPLEX_D, &DCT4_REAL_S, &DCT4_REAL_D, &DCT4_COMPLEX_S, &DCT4_COMPLEX_D, &DST4_REAL_S,
                  &DST4_REAL_D, &DST4_COMPLEX_S, &DST4_COMPLEX_D};
  int *c[44] = {&P3DFFT_EMPTY_TYPE_SINGLE, &P3DFFT_EMPTY_TYPE_DOUBLE, &P3DFFT_EMPTY_TYPE_SINGLE_COMPLEX,
                &P3DFFT_EMPTY_TYPE_DOUBLE_COMPLEX, &P3DFFT_R2CFFT_S, &P3DFFT_R2CFFT_D, &P3DFFT_C2RFFT_S,
                &P3DFFT_C2RFFT_D, &P3DFFT_CFFT_FORWARD_S, &P3DFFT_CFFT_FORWARD_D, &P3DFFT_CFFT_BACKWARD_S,
                &P3DFFT_CFFT_BACKWARD_D, &P3DFFT_DCT1_REAL_S, &P3DFFT_DCT1_REAL_D, &P3DFFT_DCT1_COMPLEX_S,
                &P3DFFT_DCT1_COMPLEX_D, &P3DFFT_DST1_REAL_S, &P3DFFT_DST1_REAL_D, &P3DFFT_DST1_COMPLEX_S,
                &P3DFFT_DST1_COMPLEX_D, &P3DFFT_DCT2_REAL_S, &P3DFFT_DCT2_REAL_D, &P3DFFT_DCT2_COMPLEX_S,
                &P3DFFT_DCT2_COMPLEX_D, &P3DFFT_DST2_REAL_S, &P3DFFT_DST2_REAL_D, &P3DFFT_DST2_COMPLEX_S,
                &P3DFFT_DST2_COMPLEX_D, &P3DFFT_DCT3_REAL_S, &P3DFFT_DCT3_REAL_D, &P3DFFT_DCT3_COMPLEX_S,
                &P3DFFT_DCT3_COMPLEX_D, &P3DFFT_DST3_REAL_S, &P3DFFT_DST3_REAL_D, &P3DFFT_DST3_COMPLEX_S,
                &P3DFFT_DST3_COMPLEX_D, &P3DFFT_DCT4_REAL_S, &P3DFFT_DCT4_REAL_D, &P3DFFT_DCT4_COMPLEX_S,
                &P3DFFT_DCT4_COMPLEX_D, &P3DFFT_DST4_REAL_S, &P3DFFT_DST4_REAL_D, &P3DFFT_DST4_COMPLEX_S,
                &P3DFFT_DST4_COMPLEX_D};
  for (int i = 0; i < 44; i++) *cpp[i] = *c[i] = i;
}

// ------------------------------------------------------------------------------------------
// runtime state
struct GridDesc {
  int gdims[3];
  int mo[3];
  int dcs;
};
struct Stage {
  int type;
  int dim;
  GridDesc g1, g2;
  int ex_index = -1;  // position in the executed schedule (selects the stage's tuning)
};
struct Buffers {
  void *scratch[2] = {nullptr, nullptr};
  size_t scratch_bytes = 0;
  void *stage_in = nullptr, *stage_out = nullptr;
  size_t stage_in_bytes = 0, stage_out_bytes = 0;
  // per-line scales of float-float intermediate fields (one int per line of the producing stage)
  void *side[2] = {nullptr, nullptr};
  size_t side_bytes[2] = {0, 0};
  bool owned = true;  // false: scratch[] belongs to the caller (never freed or reallocated here)
  void release() {
    for (int i = 0; i < 2; i++)
      if (scratch[i] && owned) cudaFree(scratch[i]);
    for (int i = 0; i < 2; i++)
      if (side[i]) cudaFree(side[i]);
    if (stage_in) cudaFree(stage_in);
    if (stage_out) cudaFree(stage_out);
    scratch[0] = scratch[1] = stage_in = stage_out = side[0] = side[1] = nullptr;
    scratch_bytes = stage_in_bytes = stage_out_bytes = side_bytes[0] = side_bytes[1] = 0;
  }
};
// A stage's float-float intermediate links (the StageDesc ffin / ffout fields).
struct FFLink {
  int ffin = 0, ffout = 0;
  const int *sin = nullptr;
  int *sout = nullptr;
  long long mi[3] = {0, 0, 0}, mo[3] = {0, 0, 0};
};
// Per-stage kernel choice: engine (Engine) and tile-dim flag, 0/0 = heuristic.
struct StageTune {
  int engine = 0, talt = 0;
  float ms = 0.f;  // measured duration when chosen by the autotuner
};
struct Plan {
  std::vector<Stage> st;  // the reference planner's stage list (reported, tested for parity)
  std::vector<Stage> ex;  // the schedule the executor runs (same transforms, see optimize_schedule)
  int L[3] = {0, 1, 2};
  int dt1 = 1, dt2 = 1, prec = 8;
  GridDesc g1, g2;
  Buffers buf;
  std::vector<StageTune> tune;  // empty: heuristic for every stage
  int tuned_arith = -1;         // FP64 arithmetic the tuning was made for
  bool live = true;
};

static std::mutex g_mu;
static std::vector<Plan *> g_plans3, g_plans1;
struct Type3 {
  int types[3];
  int prec;
};
static std::vector<Type3> g_types3d;
struct PGridRec {
  int pdims[3];
  MPI_Comm comm;
  bool live;
};
static std::vector<PGridRec> g_pgrids;
struct DGridRec {
  GridDesc g;
  int pgrid;
  int dmap[3];
};
static std::vector<DGridRec> g_dgrids;

static cudaStream_t g_stream = 0;
static int g_sync = 1;

// Execution context of the calling thread.  The batch executor runs plans on its own branch
// streams with one scratch set per branch, and records them into a CUDA graph; outside a batch
// the context is empty and the library stream, the plan's own buffers and g_sync apply.
struct ExecCtx {
  cudaStream_t st;
  Buffers *buf;
  bool capturing;                  // no synchronising call may be made
  std::vector<StageLaunch> *rec;   // non-null: record the stages instead of launching them
};
static thread_local const ExecCtx *t_ctx = nullptr;
static cudaStream_t cur_stream() { return t_ctx ? t_ctx->st : g_stream; }
static bool in_capture() { return t_ctx && t_ctx->capturing; }
static int g_arith = -1;
static DeviceTables *g_tabs = nullptr;
static std::atomic<long long> g_kcount(0);
static bool g_timers_on = false;
static double g_timer[6] = {0, 0, 0, 0, 0, 0};
static int g_device_ok = -1;

static bool ensure_device() {
  if (g_device_ok == 1) return true;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= 0) {
    cudaGetLastError();
    set_err(E_NO_DEVICE, "no CUDA device is available (%s); this library has no CPU path",
            e != cudaSuccess ? cudaGetErrorString(e) : "device count 0");
    return false;
  }
  g_device_ok = 1;
  if (!g_tabs) g_tabs = tables_create();
  return true;
}

static int arith_mode() {
  if (g_arith < 0) {
    // float-float unless P3DFFT_GB300_FP64_ARITH selects native DFMA ("0" / "native")
    const char *s = getenv("P3DFFT_GB300_FP64_ARITH");
    g_arith = (s && (s[0] == '0' || s[0] == 'n' || s[0] == 'N')) ? AR_NATIVE : AR_DF;
  }
  return g_arith;
}

// Reference-compatible behaviour for two reference defects that give deterministic results
// (on by default, so that outputs are the reference's; P3DFFT_GB300_REFERENCE_COMPAT=0 or
// p3dfft_gb300_set_reference_compat(0) selects the corrected behaviour):
//  - compute_deriv differentiates along storage axis imo[idir] (the logical dim whose storage
//    rank is idir, build/deriv.C:89-93), not along the storage axis of logical dim idir; the two
//    differ only for the 3-cycle memory orders (1,2,0) and (2,0,1);
//  - a 1D plan whose input and output orders both have the transform dim non-leading reads its
//    input as if stored in order swap0(mo1, dim): find_m overwrites the plan's own mo1
//    (build/templ.C:1015-1023) and exec then reorders from that order (exec.C:582-611).
static int g_ref_compat = -1;
static int ref_compat() {
  if (g_ref_compat < 0) {
    const char *s = getenv("P3DFFT_GB300_REFERENCE_COMPAT");
    g_ref_compat = (s && s[0] == '0') ? 0 : 1;
  }
  return g_ref_compat;
}

static long long elems(const GridDesc &g) { return (long long)g.gdims[0] * g.gdims[1] * g.gdims[2]; }

static void strides(const GridDesc &g, long long s[3]) {
  for (int i = 0; i < 3; i++) {
    s[i] = 1;
    for (int j = 0; j < 3; j++)
      if (g.mo[j] < g.mo[i]) s[i] *= g.gdims[j];
  }
}

static bool valid_mo(const int mo[3]) {
  int seen = 0;
  for (int i = 0; i < 3; i++) {
    if (mo[i] < 0 || mo[i] > 2) return false;
    seen |= 1 << mo[i];
  }
  return seen == 7;
}

static bool valid_grid(const GridDesc &g) {
  for (int i = 0; i < 3; i++)
    if (g.gdims[i] <= 0) return false;
  return valid_mo(g.mo) && g.dcs >= -1 && g.dcs <= 2;
}

// ------------------------------------------------------------------------------------------
// planner (templ.C), specialised to one task on a 1x1x1 processor grid: Pdims == 1 in every
// dim, ProcGrid::nd == 1 (init.C:1634-1641) and DataGrid::L == {0,1,2} (init.C:1813-1818)

// swap0, templ.C:816-858
static void swap0(int newmo[3], const int mo[3], int L) {
  int t[3] = {mo[0], mo[1], mo[2]};
  if (t[L] == 1) {
    int j = 0;
    while (j < 3 && t[j] != 0) j++;
    t[j] = 1;
    t[L] = 0;
  } else if (t[L] == 2) {
    for (int i = 0; i < 3; i++) t[i] = (t[i] + 1) % 3;
  }
  for (int i = 0; i < 3; i++) newmo[i] = t[i];
}

// excl, templ.C:872-882
static int excl(int a, int b) {
  if (a * b == 0) return std::max(a, b) == 1 ? 2 : 1;
  return 0;
}

// find_order, templ.C:627-802 (numtasks == 1 branch)
static bool find_order(const int types[3], const GridDesc &g1, const GridDesc &g2, int L[3]) {
  L[0] = L[1] = L[2] = -1;
  bool ok = true;
  for (int i = 0; i < 3; i++) {
    const TypeInfo &t = g_types[types[i]];
    if (t.dt1 < t.dt2) {
      if (L[0] >= 0) ok = false;
      else L[0] = i;
    } else if (t.dt1 > t.dt2) {
      if (L[2] >= 0) ok = false;
      else L[2] = i;
    }
  }
  if (L[0] >= 0 && L[2] >= 0) ok = false;
  if (L[0] < 0) {
    L[0] = 0;
    if (L[2] < 0) {
      if (g1.mo[0] > g1.mo[1]) L[0] = 1;
    } else if (L[0] == L[2]) {
      L[0] = 1;
    }
  }
  if (L[2] < 0) {
    for (int i = 0; i < 3; i++)
      if (g2.mo[i] == 0) L[2] = i;
    if (L[2] == L[0]) L[2] = (L[0] + 1) % 3;
  }
  L[1] = excl(L[0], L[2]);
  return ok;
}

static int empty_type(int dt, int prec) { return dt == 2 ? (prec == 4 ? 2 : 3) : (prec == 4 ? 0 : 1); }

static void optimize_schedule(Plan *P);

// transform3D ctor stage loop, templ.C:224-420
static Plan *make_plan3(const int types[3], const GridDesc &g1, const GridDesc &g2) {
  for (int i = 0; i < 3; i++)
    if (types[i] < 0 || types[i] >= 44) {
      set_err(E_BAD_ARG, "transform type %d is undefined", types[i]);
      return nullptr;
    }
  if (!valid_grid(g1) || !valid_grid(g2)) {
    set_err(E_BAD_ARG, "invalid grid description (dims must be > 0, memory order a permutation of 0,1,2)");
    return nullptr;
  }
  Plan *P = new Plan();
  P->g1 = g1;
  P->g2 = g2;
  if (!find_order(types, g1, g2, P->L)) {
    set_err(E_PLAN, "transform3D: more than one R2C or C2R 1D transform, or both (templ.C:640-658)");
    delete P;
    return nullptr;
  }
  const TypeInfo &t0 = g_types[types[P->L[0]]];
  P->dt1 = t0.dt1;
  P->prec = t0.prec;
  int monext[3] = {g1.mo[0], g1.mo[1], g1.mo[2]}, mocurr[3];
  int gd[3] = {g1.gdims[0], g1.gdims[1], g1.gdims[2]};
  int dcs = g1.dcs, dt_prev = t0.dt1;
  for (int s = 0; s < 3; s++) {
    const int Ls = P->L[s];
    const TypeInfo &t = g_types[types[Ls]];
    if (t.prec != P->prec) {
      set_err(E_PLAN, "transform3D: 1D transform types of different precision");
      delete P;
      return nullptr;
    }
    if (t.dt1 != dt_prev) {
      set_err(E_PLAN, "transform3D: datatypes don't match between stages (%d %d)", t.dt1, dt_prev);
      delete P;
      return nullptr;
    }
    for (int i = 0; i < 3; i++) mocurr[i] = monext[i];
    Stage st;
    st.type = types[Ls];
    st.dim = Ls;
    st.g1 = GridDesc{{gd[0], gd[1], gd[2]}, {mocurr[0], mocurr[1], mocurr[2]}, dcs};
    if (t.dt1 < t.dt2) {  // R2C
      dcs = Ls;
      gd[dcs] = gd[dcs] / 2 + 1;
    } else if (t.dt2 < t.dt1) {  // C2R
      if (dcs < 0) {
        set_err(E_PLAN, "transform3D: complex-to-real stage but the input grid has no conjugate-symmetric dim");
        delete P;
        return nullptr;
      }
      gd[dcs] = (gd[dcs] - 1) * 2;
      dcs = -1;
    }
    if (s < 2) {
      if (t.kind != K_EMPTY) swap0(monext, mocurr, Ls);
    } else {
      for (int i = 0; i < 3; i++) monext[i] = g2.mo[i];
      if (monext[Ls] != 0) swap0(monext, mocurr, Ls);
    }
    st.g2 = GridDesc{{gd[0], gd[1], gd[2]}, {monext[0], monext[1], monext[2]}, dcs};
    P->st.push_back(st);
    dt_prev = t.dt2;
  }
  P->dt2 = dt_prev;
  for (int i = 0; i < 3; i++)
    if (gd[i] != g2.gdims[i]) {
      set_err(E_PLAN, "transform3D: output grid dims (%d %d %d) do not match the transform (%d %d %d)", g2.gdims[0],
              g2.gdims[1], g2.gdims[2], gd[0], gd[1], gd[2]);
      delete P;
      return nullptr;
    }
  if (monext[0] != g2.mo[0] || monext[1] != g2.mo[1] || monext[2] != g2.mo[2]) {  // final_seq
    Stage st;
    const GridDesc &prev = P->st.back().g2;
    int td = 0;
    if (prev.mo[td] != 0 && g2.mo[td] != 0) td = 1;
    st.type = empty_type(P->dt2, P->prec);
    st.dim = td;
    st.g1 = prev;
    st.g2 = g2;
    P->st.push_back(st);
  }
  optimize_schedule(P);
  for (size_t i = 0; i < P->ex.size(); i++) P->ex[i].ex_index = (int)i;
  return P;
}

// ------------------------------------------------------------------------------------------
// Execution schedule.  The reference planner fixes the order of the 1D transforms and every
// intermediate memory order (templ.C:224-420).  The result of the 3D transform depends only on the
// input and output grids and on the 1D transform each dim gets: the intermediate layouts are
// internal, and separable transforms commute (R2C must come first and C2R last, where the data
// type changes).  On GB300 a stage whose lines are spread far apart in memory (a transform dim of
// stride >= 16 Ki elements read or written through the tile dim) streams at ~70% of the rate of a
// stage with contiguous lines, so the executor picks, over all admissible orders and the 36
// choices of the two intermediate memory orders, the schedule with the cheapest accesses, keeping
// the reference schedule on ties.  P3DFFT_GB300_REFERENCE_SCHEDULE=1 runs the reference schedule.
// Cost of one side of a stage: 1 for contiguous lines, or for lines taken across a contiguous
// tile dim t with the line's points near each other; 1.4 with the points >= 16 Ki elements
// apart; 4 when neither the lines nor t are contiguous (uncoalesced).  Plus 0.15 when rows of the
// contiguous dim are not a multiple of 128 bytes (e.g. 257 complex values), so that accesses
// straddle an extra cache line (measured: the float-float C2R stage reading 257-element rows
// ran 0.14 ms, 13%, slower than reading 512-element rows).
static double side_cost(const long long s[3], const int *gd, int L, int t, int esz) {
  double c;
  int cdim;
  if (s[L] == 1) {
    c = 1.0;
    cdim = L;
  } else if (s[t] != 1) {
    return 4.0;
  } else {
    c = s[L] >= 16384 ? 1.4 : 1.0;
    cdim = t;
  }
  return c + (((long long)gd[cdim] * esz) % 128 ? 0.15 : 0.0);
}

// Load + store cost of a stage with the kernel's choice of tile dim (launch_stage): by output
// stride when the input lines are contiguous, else by input stride.
static double stage_cost(const Stage &st, int prec) {
  long long s1[3], s2[3];
  strides(st.g1, s1);
  strides(st.g2, s2);
  const TypeInfo &ti = g_types[st.type];
  const int L = st.dim, a = (L + 1) % 3, b = (L + 2) % 3;
  const int t = (s1[L] == 1) ? (s2[a] <= s2[b] ? a : b) : (s1[a] <= s1[b] ? a : b);
  return side_cost(s1, st.g1.gdims, L, t, ti.dt1 * prec) + side_cost(s2, st.g2.gdims, L, t, ti.dt2 * prec);
}

static double schedule_cost(const std::vector<Stage> &v, int prec) {
  double c = 0;
  for (auto &st : v)
    if (g_types[st.type].kind != K_EMPTY) c += stage_cost(st, prec);
  return c;
}

static void optimize_schedule(Plan *P) {
  P->ex = P->st;
  const char *ref = getenv("P3DFFT_GB300_REFERENCE_SCHEDULE");
  if ((ref && ref[0] == '1') || P->st.size() != 3) return;
  for (auto &st : P->st)
    if (g_types[st.type].kind == K_EMPTY) return;
  static const int MO[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  static const int PERM[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  double best = schedule_cost(P->ex, P->prec) - 1e-9;
  for (auto &pm : PERM) {
    // the data type must chain: real-to-complex first, complex-to-real last
    int dt = P->dt1;
    bool ok = true;
    for (int k = 0; k < 3 && ok; k++) {
      const TypeInfo &t = g_types[P->st[pm[k]].type];
      ok = t.dt1 == dt;
      dt = t.dt2;
    }
    if (!ok) continue;
    for (int a = 0; a < 6; a++)
      for (int b = 0; b < 6; b++) {
        std::vector<Stage> v(3);
        GridDesc cur = P->g1;
        for (int k = 0; k < 3; k++) {
          const Stage &rs = P->st[pm[k]];
          const TypeInfo &t = g_types[rs.type];
          Stage st = rs;
          st.g1 = cur;
          GridDesc nx = cur;
          if (t.dt1 < t.dt2) {  // R2C
            nx.dcs = rs.dim;
            nx.gdims[rs.dim] = nx.gdims[rs.dim] / 2 + 1;
          } else if (t.dt2 < t.dt1) {  // C2R
            nx.gdims[rs.dim] = (nx.gdims[rs.dim] - 1) * 2;
            nx.dcs = -1;
          }
          const int *mo = k == 0 ? MO[a] : (k == 1 ? MO[b] : P->g2.mo);
          for (int i = 0; i < 3; i++) nx.mo[i] = mo[i];
          if (k == 2) nx = P->g2;
          st.g2 = nx;
          v[k] = st;
          cur = nx;
        }
        bool dims_ok = true;
        for (int i = 0; i < 3; i++) dims_ok &= v[2].g2.gdims[i] == P->g2.gdims[i];
        if (!dims_ok) continue;
        const double c = schedule_cost(v, P->prec);
        if (c < best) {
          best = c - 1e-9;
          P->ex = v;
        }
      }
  }
}

static Plan *make_plan1(int type, const GridDesc &g1, const GridDesc &g2, int d) {
  if (type < 0 || type >= 44 || d < 0 || d > 2) {
    set_err(E_BAD_ARG, "transplan: undefined type %d or dimension %d", type, d);
    return nullptr;
  }
  if (!valid_grid(g1) || !valid_grid(g2)) {
    set_err(E_BAD_ARG, "transplan: invalid grid description");
    return nullptr;
  }
  const TypeInfo &t = g_types[type];
  int a = (d + 1) % 3, b = (d + 2) % 3;
  if (g1.gdims[a] != g2.gdims[a] || g1.gdims[b] != g2.gdims[b]) {
    set_err(E_PLAN, "transplan: grids differ outside the transform dimension");
    return nullptr;
  }
  int n1 = g1.gdims[d], n2 = g2.gdims[d];
  bool ok = (t.kind == K_R2C) ? (n2 == n1 / 2 + 1) : (t.kind == K_C2R) ? (n1 == n2 / 2 + 1) : (n1 == n2);
  if (!ok) {
    set_err(E_PLAN, "transplan: dimension %d sizes %d -> %d do not fit the transform type", d, n1, n2);
    return nullptr;
  }
  Plan *P = new Plan();
  P->g1 = g1;
  P->g2 = g2;
  // find_m (templ.C:1015-1023): neither order leads with the transform dim, so the reference
  // replaces its input order by swap0(mo1, d) and reads the input in that order
  if (ref_compat() && t.kind != K_EMPTY && g1.mo[d] != 0 && g2.mo[d] != 0) swap0(P->g1.mo, g1.mo, d);
  P->dt1 = t.dt1;
  P->dt2 = t.dt2;
  P->prec = t.prec;
  Stage st;
  st.type = type;
  st.dim = d;
  st.g1 = P->g1;
  st.g2 = g2;
  P->st.push_back(st);
  P->ex = P->st;
  P->ex[0].ex_index = 0;
  return P;
}

// ------------------------------------------------------------------------------------------
// executor
static bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host arrays read (bit 0) / written (bit 1) by the first / last stage directly over
// NVLink-C2C instead of staged through HBM.  -1: from P3DFFT_GB300_HOST_DIRECT at first use
// ("0" none, "in", "out", anything else both; default both).
// Pipelining of the host-link-bound end stages with their neighbour stage (default on;
// P3DFFT_GB300_PIPELINE=0 or p3dfft_gb300_set_host_pipeline(0) turns it off)
static int g_host_pipe = -1;
static bool pipeline_host_stages() {
  if (g_host_pipe < 0) {
    const char *e = getenv("P3DFFT_GB300_PIPELINE");
    g_host_pipe = (e && e[0] == '0') ? 0 : 1;
  }
  return g_host_pipe == 1;
}
// Grid cap of an end stage that reads / writes a host array in place while its
// neighbour stage runs beside it slab by slab (0: no such pipelining).  -1 (default): from
// P3DFFT_GB300_LINK_CTAS when set, else one CTA per SM for FP64 stages and two for FP32.
// Measured on the 512^3 round trip (forward / backward ms, +-0.05 between runs): FP64 38 CTAs
// 22.7 ms in all, 76 13.6, 152 6.13 / 6.75, 228 6.25 / 6.74, 304 6.45 / 6.71, stage after stage
// 6.59 / 7.02; FP32 152 2.92 / 3.16, 304 2.86 / 3.13, 456 2.88 / 3.14, stage after stage
// 2.99 / 3.22.
static int g_link_ctas = -1;
static int link_ctas_set() {  // the explicit cap, or -1
  if (g_link_ctas < 0) {
    const char *e = getenv("P3DFFT_GB300_LINK_CTAS");
    if (e) return std::max(0, atoi(e));
  }
  return g_link_ctas;
}
static int link_ctas(int prec) {
  const int n = link_ctas_set();
  if (n >= 0) return n;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      sms = 0;
      return 0;  // asked again at the next call
    }
  }
  return sms * (prec == 4 ? 2 : 1);
}
// Tile counters for the link stage's persistent CTAs (P3DFFT_GB300_TILE_CTR=0: fixed grid stride)
static bool tile_ctr_on() {
  static int on = -1;
  if (on < 0) {
    const char *e = getenv("P3DFFT_GB300_TILE_CTR");
    on = (e && e[0] == '0') ? 0 : 1;
  }
  return on == 1;
}
static int g_host_direct = -1;
static int host_direct_mode() {
  if (g_host_direct < 0) {
    const char *e = getenv("P3DFFT_GB300_HOST_DIRECT");
    g_host_direct = !e ? 3 : (e[0] == '0' ? 0 : (!strcmp(e, "in") ? 1 : (!strcmp(e, "out") ? 2 : 3)));
  }
  return g_host_direct;
}
// Pageable host memory read / written by the kernels in place: only where the device accesses
// pageable memory coherently through the host's page tables (address translation over
// NVLink-C2C, as on Grace; cudaDevAttrPageableMemoryAccessUsesHostPageTables), not where access
// would migrate pages.  -1: P3DFFT_GB300_PAGEABLE_DIRECT at first use ("0" off; default off).
static int g_pageable_direct = -1;
static int pageable_access_ok() {  // 1: the device reads pageable memory through the host's tables
  static int ok = -1;
  if (ok < 0) {
    int dev = 0, pm = 0, hpt = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pm, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    ok = pm && hpt ? 1 : 0;
  }
  return ok;
}
static bool pageable_direct() {
  if (g_pageable_direct < 0) {
    const char *e = getenv("P3DFFT_GB300_PAGEABLE_DIRECT");
    g_pageable_direct = (e && e[0] == '1') ? 1 : 0;
  }
  return g_pageable_direct == 1 && pageable_access_ok() == 1;
}
// Page-locked host memory (cudaHostAlloc / cudaHostRegister) is addressable by kernels over
// NVLink-C2C; returns its device-side address (pageable memory: the pointer itself when
// pageable_direct()), or nullptr for any other pointer.
static void *mapped_host_ptr(const void *p) {
  if (!p || !host_direct_mode()) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  if (a.type == cudaMemoryTypeUnregistered && pageable_direct()) return const_cast<void *>(p);
  return nullptr;
}

static bool ensure_buf(void **p, size_t *have, size_t need) {
  if (*have >= need && *p) return true;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  if (cudaMalloc(p, need) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_err(E_CUDA, "cudaMalloc of %zu bytes failed", need);
    return false;
  }
  *have = need;
  return true;
}

static size_t stage_out_bytes(const Plan *P, const Stage &s) {
  const TypeInfo &t = g_types[s.type];
  return (size_t)elems(s.g2) * t.dt2 * P->prec;
}

struct TimerScope {
  cudaEvent_t a = nullptr, b = nullptr;
  int phase;
  explicit TimerScope(int ph) : phase(ph) {
    if (!g_timers_on || t_ctx) return;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, cur_stream());
  }
  ~TimerScope() {
    if (!g_timers_on || !a) return;
    cudaEventRecord(b, cur_stream());
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    g_timer[phase] += ms * 1e-3;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

static void fill_stage_desc(const Plan *P, const Stage &s, bool deriv, StageDesc &d) {
  const TypeInfo &t = g_types[s.type];
  d.kind = t.kind;
  d.r2r = t.r2r;
  d.prec = P->prec;
  d.dt1 = t.dt1;
  d.dt2 = t.dt2;
  d.L = s.dim;
  for (int i = 0; i < 3; i++) {
    d.d1[i] = s.g1.gdims[i];
    d.d2[i] = s.g2.gdims[i];
  }
  strides(s.g1, d.s1);
  strides(s.g2, d.s2);
  d.deriv = deriv ? 1 : 0;
  const size_t idx = (size_t)s.ex_index;
  d.engine = d.talt = 0;
  if (s.ex_index >= 0 && P->tune.size() == P->ex.size() && idx < P->ex.size() &&
      (P->prec == 4 || P->tuned_arith == arith_mode())) {
    d.engine = P->tune[idx].engine;
    d.talt = P->tune[idx].talt;
  }
}

// A sub-box of a stage: coordinates [c, c + m) along dim sd, in the stage's full input and output
// layouts (the strides of the whole field).
struct SlabBox {
  int sd, c, m;
  int ctas = 0;            // the stage's grid cap (StageDesc::max_ctas)
  int *ctr = nullptr;      // and its zeroed tile counter (StageDesc::tile_ctr)
};

// engine_override >= 0 replaces the plan's tuned engine choice for this stage (0 = heuristic);
// ff: float-float intermediate links of this stage; box: run only that sub-box of the stage
static int run_stage(const Plan *P, const Stage &s, const void *src, void *dst, bool deriv,
                     const void *tw_given = nullptr, const void *aux_given = nullptr, int engine_override = -1,
                     const FFLink *ff = nullptr, const SlabBox *box = nullptr) {
  const TypeInfo &t = g_types[s.type];
  if (t_ctx && t_ctx->rec) {  // recording for a grouped launch set
    StageLaunch sl;
    fill_stage_desc(P, s, deriv, sl.d);
    sl.src = src;
    sl.dst = dst;
    sl.arith = P->prec == 8 ? arith_mode() : AR_NATIVE;
    t_ctx->rec->push_back(sl);
    return E_OK;
  }
  int launched = 0;
  int rc = E_OK;
  if (t.kind == K_EMPTY) {
    bool same = s.g1.mo[0] == s.g2.mo[0] && s.g1.mo[1] == s.g2.mo[1] && s.g1.mo[2] == s.g2.mo[2];
    size_t bytes = (size_t)elems(s.g1) * t.dt1 * P->prec;
    TimerScope ts(2);
    if (same) {
      if (src != dst && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, cur_stream()) != cudaSuccess)
        rc = E_CUDA;
    } else {
      long long s1[3], s2[3];
      strides(s.g1, s1);
      strides(s.g2, s2);
      rc = launch_permute(s.g1.gdims, s1, s2, t.dt1 * P->prec, src, dst, cur_stream(), &launched);
    }
  } else {
    StageDesc d;
    fill_stage_desc(P, s, deriv, d);
    if (engine_override >= 0) d.engine = engine_override;
    if (ff) {
      d.ffin = ff->ffin;
      d.ffout = ff->ffout;
      d.sin = ff->sin;
      d.sout = ff->sout;
      for (int i = 0; i < 3; i++) {
        d.mi[i] = ff->mi[i];
        d.mo[i] = ff->mo[i];
      }
    }
    if (box) {  // the sub-box keeps the full field's strides; buffers and scale arrays are offset
      const int sd = box->sd;
      src = static_cast<const unsigned char *>(src) + (size_t)box->c * d.s1[sd] * t.dt1 * P->prec;
      dst = static_cast<unsigned char *>(dst) + (size_t)box->c * d.s2[sd] * t.dt2 * P->prec;
      d.d1[sd] = d.d2[sd] = box->m;
      d.max_ctas = box->ctas;
      d.tile_ctr = box->ctr;
      if (d.sin) d.sin += (long long)box->c * d.mi[sd];
      if (d.sout) d.sout += (long long)box->c * d.mo[sd];
    }
    bool reorder = !(s.g1.mo[0] == s.g2.mo[0] && s.g1.mo[1] == s.g2.mo[1] && s.g1.mo[2] == s.g2.mo[2]);
    TimerScope ts(deriv ? 3 : (reorder ? 1 : 0));
    rc = launch_stage(d, src, dst, P->prec == 8 ? arith_mode() : AR_NATIVE, cur_stream(), g_tabs, &launched, tw_given,
                      aux_given);
  }
  g_kcount += launched;
  if (rc != E_OK) {
    if (rc == E_CUDA) set_err(E_CUDA, "kernel launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    else if (rc == E_TOO_LARGE) set_err(E_TOO_LARGE, "transform length or grid too large for this release");
    else if (rc == E_UNSUPPORTED) set_err(E_UNSUPPORTED, "unsupported transform size/type combination");
    else if (rc == E_ALIGN)
      set_err(E_ALIGN, "data pointers must be aligned to one complex element (16 bytes FP64, 8 bytes FP32)");
    else set_err(rc, "invalid stage description");
  }
  return rc;
}

// A dim that is the slowest of both the stage's input and output layouts and not its transform
// dim: slabs along it are contiguous on both sides and the other dims' strides do not depend on it.
static int slab_dim(const Stage &st) {
  if (g_types[st.type].kind == K_EMPTY) return -1;
  for (int d = 0; d < 3; d++)
    if (d != st.dim && st.g1.mo[d] == 2 && st.g2.mo[d] == 2 && st.g1.gdims[d] >= 2) return d;
  return -1;
}

static cudaStream_t g_copy_stream = nullptr;
constexpr int kMaxSlabs = 16;
static cudaEvent_t g_slab_ev[2 * kMaxSlabs + 1];  // per slab in, per slab out, and the join

// Runs one stage slab by slab along dim sd, overlapping the host copy of each slab on the copy
// stream: side 0 copies host `host` into `src` (the stage's staged input) slab by slab before
// the stage reads it; side 1 copies the stage's output `dst` to host `host` slab by slab after
// the stage writes it.  All work is ordered on the library stream when this returns.
// The float-float links of the slab starting at coordinate c along dim sd: the scale arrays are
// indexed by global coordinates, the slab's lines by coordinates within the slab.
static const FFLink *slab_link(const FFLink *ff, int c, int sd, FFLink *out) {
  if (!ff) return nullptr;
  *out = *ff;
  if (out->sin) out->sin += (long long)c * out->mi[sd];
  if (out->sout) out->sout += (long long)c * out->mo[sd];
  return out;
}

static int ensure_copy_stream() {
  if (!g_copy_stream) {
    for (auto &e : g_slab_ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return E_CUDA;
    if (cudaStreamCreateWithFlags(&g_copy_stream, cudaStreamNonBlocking) != cudaSuccess) return E_CUDA;
  }
  return E_OK;
}

static int run_stage_slabs(const Plan *P, const Stage &st, int sd, const void *host, const void *src, void *dst,
                           bool deriv, int side, const FFLink *ff = nullptr) {
  const int NS = 8;
  if (ensure_copy_stream() != E_OK) return E_CUDA;
  const TypeInfo &t = g_types[st.type];
  long long s1[3], s2[3];
  strides(st.g1, s1);
  strides(st.g2, s2);
  const size_t u1 = (size_t)s1[sd] * t.dt1 * P->prec, u2 = (size_t)s2[sd] * t.dt2 * P->prec;  // bytes per slab row
  const int len = st.g1.gdims[sd];
  int f = 1;  // slab starts stay 16-byte aligned on both sides
  while (f < 16 && ((f * u1) % 16 || (f * u2) % 16)) f++;
  const int per = ((len + NS - 1) / NS + f - 1) / f * f;
  cudaStream_t cs = g_copy_stream, ms = cur_stream();
  // the copy stream starts after everything already queued on the library stream
  if (cudaEventRecord(g_slab_ev[2 * kMaxSlabs], ms) != cudaSuccess ||
      cudaStreamWaitEvent(cs, g_slab_ev[2 * kMaxSlabs], 0) != cudaSuccess)
    return E_CUDA;
  int rc = E_OK;
  FFLink sff;
  for (int c = 0, k = 0; c < len && rc == E_OK; c += per, k++) {
    const int m = std::min(per, len - c);
    Stage sl = st;
    sl.g1.gdims[sd] = sl.g2.gdims[sd] = m;
    const unsigned char *sp = static_cast<const unsigned char *>(src) + (size_t)c * u1;
    unsigned char *dp = static_cast<unsigned char *>(dst) + (size_t)c * u2;
    if (side == 0) {
      if (cudaMemcpyAsync(const_cast<unsigned char *>(sp), static_cast<const unsigned char *>(host) + (size_t)c * u1,
                          (size_t)m * u1, cudaMemcpyHostToDevice, cs) != cudaSuccess ||
          cudaEventRecord(g_slab_ev[k], cs) != cudaSuccess || cudaStreamWaitEvent(ms, g_slab_ev[k], 0) != cudaSuccess)
        return E_CUDA;
      rc = run_stage(P, sl, sp, dp, deriv, nullptr, nullptr, -1, slab_link(ff, c, sd, &sff));
    } else {
      rc = run_stage(P, sl, sp, dp, deriv, nullptr, nullptr, -1, slab_link(ff, c, sd, &sff));
      if (rc == E_OK &&
          (cudaEventRecord(g_slab_ev[k], ms) != cudaSuccess || cudaStreamWaitEvent(cs, g_slab_ev[k], 0) != cudaSuccess ||
           cudaMemcpyAsync(static_cast<unsigned char *>(const_cast<void *>(host)) + (size_t)c * u2, dp, (size_t)m * u2,
                           cudaMemcpyDeviceToHost, cs) != cudaSuccess))
        return E_CUDA;
    }
  }
  if (side == 1) {  // the library stream continues after the last copy
    if (cudaEventRecord(g_slab_ev[2 * kMaxSlabs], cs) != cudaSuccess ||
        cudaStreamWaitEvent(ms, g_slab_ev[2 * kMaxSlabs], 0) != cudaSuccess)
      return E_CUDA;
  }
  return rc;
}

// ------------------------------------------------------------------------------------------
// Autotuner.  For every stage of a plan it times each kernel choice the stage admits — the
// specialised kernel (compile-time radix plan and tile shape), the register engine (power-of-two
// lengths, tile lines chosen at run time), the generic mixed-radix engine — each with the tile's
// consecutive lines taken along either batch dim, and keeps the fastest.  Choices are cached by
// stage (transform kind, precision, FP64 arithmetic, dims and strides in and out), so a plan's key
// (grid, transform types, dtype) decomposes into its stages' keys and plans sharing a stage share
// its tuning; the cache can be saved to and loaded from a text file.
static std::mutex g_tmu;
static std::map<std::string, StageTune> g_tune_cache;
static bool g_autotune = false;

static std::string stage_key(const StageDesc &d, int arith) {
  char b[400];
  snprintf(b, sizeof b, "%d %d %d %d %d %d %d %d %d %d %d %d %d %lld %lld %lld %lld %lld %lld", d.kind, d.r2r, d.prec,
           d.prec == 8 ? arith : 0, d.dt1, d.dt2, d.L, d.d1[0], d.d1[1], d.d1[2], d.d2[0], d.d2[1], d.d2[2], d.s1[0],
           d.s1[1], d.s1[2], d.s2[0], d.s2[1], d.s2[2]);
  return b;
}

static int autotune_plan(Plan *P) {
  if (!ensure_device()) return t_err;
  const int n = (int)P->ex.size();
  const int arith = arith_mode();
  const int ar = P->prec == 8 ? arith : AR_NATIVE;
  std::vector<StageTune> tune(n);
  size_t maxb = 0;
  for (auto &s : P->ex) {
    const TypeInfo &t = g_types[s.type];
    maxb = std::max(maxb, std::max((size_t)elems(s.g1) * t.dt1, (size_t)elems(s.g2) * t.dt2) * P->prec);
  }
  void *bi = nullptr, *bo = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = E_OK;
  P->tune.clear();  // fill_stage_desc below must see the heuristic
  for (int si = 0; si < n && rc == E_OK; si++) {
    const Stage &s = P->ex[si];
    if (g_types[s.type].kind == K_EMPTY) continue;
    StageDesc d;
    fill_stage_desc(P, s, false, d);
    const std::string key = stage_key(d, arith);
    {
      std::lock_guard<std::mutex> g(g_tmu);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        tune[si] = it->second;
        continue;
      }
    }
    if (!bi) {
      if (cudaMalloc(&bi, maxb) != cudaSuccess || cudaMalloc(&bo, maxb) != cudaSuccess ||
          cudaMemset(bi, 0, maxb) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
          cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        set_err(E_CUDA, "autotune: buffer allocation failed");
        rc = E_CUDA;
        break;
      }
    }
    StageTune best;
    best.ms = 1e30f;
    for (int e : {ENG_FAST, ENG_FIXED, ENG_GENERIC, ENG_BLUESTEIN}) {
      for (int ta = 0; ta < 2; ta++) {
        d.engine = e;
        d.talt = ta;
        if (launch_stage(d, bi, bo, ar, g_stream, g_tabs, nullptr) != E_OK) {  // not admissible
          cudaGetLastError();
          continue;
        }
        // repeat until ~0.3 ms of work is timed (at least 3, at most 50 launches)
        float ms = 0.f;
        int reps = 3;
        for (int round = 0; round < 2; round++) {
          cudaEventRecord(e0, g_stream);
          for (int r = 0; r < reps; r++) launch_stage(d, bi, bo, ar, g_stream, g_tabs, nullptr);
          cudaEventRecord(e1, g_stream);
          cudaEventSynchronize(e1);
          cudaEventElapsedTime(&ms, e0, e1);
          ms /= reps;
          if (round == 0 && ms > 0.f) reps = std::max(3, std::min(50, (int)(0.3f / ms)));
        }
        if (ms < best.ms) {
          best.engine = e;
          best.talt = ta;
          best.ms = ms;
        }
      }
    }
    if (best.ms >= 1e30f) best = StageTune();  // nothing ran: keep the heuristic
    tune[si] = best;
    std::lock_guard<std::mutex> g(g_tmu);
    g_tune_cache[key] = best;
  }
  if (bi) cudaFree(bi);
  if (bo) cudaFree(bo);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc != E_OK) return rc;
  P->tune = tune;
  P->tuned_arith = arith;
  return E_OK;
}

// Float-float intermediate fields: between two consecutive stages that both run the specialised
// float-float kernels (C2C, or an R2C producer / C2R consumer), the producer stores its values as
// packed float-float pairs at its own per-line power-of-two scale (the scales go to a side array)
// instead of converting them to IEEE doubles, and the consumer rescales them instead of converting
// back: the same 16 bytes per complex value, without the integer-heavy conversions.  The caller
// sees IEEE doubles only: the first stage reads and the last stage writes them.
// P3DFFT_GB300_FF_INTERMEDIATE=0 or p3dfft_gb300_set_ff_intermediates(0) turns this off.
static int g_ff_inter = -1;
static bool ff_intermediates() {
  if (g_ff_inter < 0) {
    const char *e = getenv("P3DFFT_GB300_FF_INTERMEDIATE");
    g_ff_inter = (e && e[0] == '0') ? 0 : 1;
  }
  return g_ff_inter == 1;
}

// Whether the stage runs the specialised float-float kernel of a kind that can read (C2C, C2R) or
// write (C2C, R2C) float-float intermediates, with these buffers.
static void stage_ff_capable(const Plan *P, const Stage &st, const void *src, void *dst, bool deriv, bool *can_in,
                             bool *can_out) {
  *can_in = *can_out = false;
  const int k = g_types[st.type].kind;
  if (P->prec != 8 || arith_mode() != AR_DF) return;
  if (k != K_C2C_FWD && k != K_C2C_BWD && k != K_R2C && k != K_C2R) return;
  StageDesc d;
  fill_stage_desc(P, st, deriv, d);
  TableNeed need{0, 0, 0, 0};
  if (launch_stage(d, src, dst, AR_DF, cur_stream(), nullptr, nullptr, nullptr, nullptr, &need) != E_OK || !need.ff)
    return;
  *can_in = k != K_R2C;
  *can_out = k != K_C2R;
}

// Scale index of an intermediate field of grid g stored by lines along dim A: coordinate
// multipliers over the two other dims (ascending), 0 along A.
static void ff_multipliers(const GridDesc &g, int A, int B, long long m[3]) {
  // B (the consuming stage's transform dim) varies fastest, so that the consumer's loads of the
  // scales of one line's points are contiguous; its other dim is the producer's tile dim in the
  // usual schedules, so the producer's stores of its lines' scales are contiguous too
  int d1 = -1, d2 = -1;
  for (int d = 0; d < 3; d++)
    if (d != A) (d1 < 0 ? d1 : d2) = d;
  if (B == d2) std::swap(d1, d2);
  m[A] = 0;
  m[d1] = 1;
  m[d2] = g.gdims[d1];
}

// Two consecutive stages pipelined slab by slab along dim sd, which neither transforms: stage a
// runs slab k on the library stream, stage b runs slab k on a second stream as soon as that slab
// of a is written, so b works alongside a's later slabs.  Used with host staging copies (which
// bound the step): both stages then hide behind the transfer.  All work is ordered on the library
// stream when this returns.
static int pair_slab_dim(const Stage &a, const Stage &b) {
  if (g_types[a.type].kind == K_EMPTY || g_types[b.type].kind == K_EMPTY || a.dim == b.dim) return -1;
  const int sd = 3 - a.dim - b.dim;
  return a.g1.gdims[sd] >= 8 ? sd : -1;
}
static cudaStream_t g_pipe_stream = nullptr;
static cudaEvent_t g_pipe_ev[kMaxSlabs + 1];  // one per slab, and the fork / join event

// host_in: stage a's input is staged from host array host_in into src, slab k copied on the copy
// stream just before stage a's slab k; host_out: stage b's output dst is copied to host array
// host_out slab by slab as stage b finishes each (sd the slowest dim of that layout, so each slab
// is one contiguous copy).
static int ensure_copy_stream();
// link 1: stage a reads a host array in place (page-locked, or pageable with in-place access),
// link 2: stage b writes one; that stage
// bounds the pair, so it runs on the priority stream with its grid capped at link_ctas persistent
// CTAs (enough to keep the host link busy) and the other stage's slabs take the remaining SM time.
static int run_pair_slabs(const Plan *P, int s, const void *src, void *mid, void *dst, int idir, const FFLink *lka,
                          const FFLink *lkb, int sd, const void *host_in = nullptr, void *host_out = nullptr,
                          int link = 0, int link_ctas = 0) {
  static int NS = 0;  // slabs (P3DFFT_GB300_PIPE_SLABS, 2..kMaxSlabs, default 8)
  if (!NS) {
    const char *e = getenv("P3DFFT_GB300_PIPE_SLABS");
    NS = e ? std::max(2, std::min(kMaxSlabs, atoi(e))) : 8;
  }
  if (!g_pipe_stream) {
    // the second stage's slabs get the highest priority, so that each starts as soon as its slab
    // of the first stage is written rather than queueing behind that stage's later slabs
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&g_pipe_stream, cudaStreamNonBlocking, hi) != cudaSuccess) return E_CUDA;
    for (auto &e : g_pipe_ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return E_CUDA;
  }
  if ((host_in || host_out) && ensure_copy_stream() != E_OK) return E_CUDA;
  const Stage &a = P->ex[s], &b = P->ex[s + 1];
  const bool da = idir >= 0 && a.dim == idir, db = idir >= 0 && b.dim == idir;
  // slab starts stay 16-byte aligned in all four layouts
  size_t u[4];
  {
    long long s1[3], s2[3];
    strides(a.g1, s1);
    strides(a.g2, s2);
    u[0] = (size_t)s1[sd] * g_types[a.type].dt1 * P->prec;
    u[1] = (size_t)s2[sd] * g_types[a.type].dt2 * P->prec;
    strides(b.g1, s1);
    strides(b.g2, s2);
    u[2] = (size_t)s1[sd] * g_types[b.type].dt1 * P->prec;
    u[3] = (size_t)s2[sd] * g_types[b.type].dt2 * P->prec;
  }
  int f = 1;
  while (f < 16 && ((f * u[0]) % 16 || (f * u[1]) % 16 || (f * u[2]) % 16 || (f * u[3]) % 16)) f++;
  const int len = a.g1.gdims[sd];
  // Slab starts along sd.  Staged copies: NS equal slabs.  A link stage: a few large slabs and one
  // thin slab where the neighbour stage runs outside the link time (last for the forward, where
  // the neighbour follows the link stage; first for the backward, where it leads), since each
  // slab boundary stalls the link stage (its slowest CTA) and the thin slab bounds the exposed
  // neighbour work; the thin link slab must still outlast one large neighbour slab.  Measured on
  // the 512^3 FP64 round trip (large slabs, thin = len / TAILDIV): 3, 16: 12.65 ms; 4, 32: 12.74;
  // 3, 32: 12.78; 5, 32: 12.79; 3, 64: 12.87; 7, 8 (8 equal slabs): 12.93; 2, 32: 13.28.
  static int NBIG = 0, TAILDIV = 0;  // P3DFFT_GB300_LINK_SLABS (default 3), P3DFFT_GB300_LINK_TAIL (16)
  if (!NBIG) {
    const char *e1 = getenv("P3DFFT_GB300_LINK_SLABS"), *e2 = getenv("P3DFFT_GB300_LINK_TAIL");
    NBIG = e1 ? std::max(1, std::min(kMaxSlabs - 1, atoi(e1))) : 3;
    TAILDIV = e2 ? std::max(2, atoi(e2)) : 16;
  }
  auto up = [&](int v) { return (v + f - 1) / f * f; };
  std::vector<int> cuts;  // slab starts (multiples of f), then len
  const int thin = link ? up(std::max(1, len / TAILDIV)) : 0;
  // the large slabs cover [lo, hi); the thin one [0, lo) (backward) or [hi, len) (forward)
  const int lo = link == 2 ? thin : 0, hi = link == 1 ? (len - thin) / f * f : len;
  if (link && thin < len && hi - lo >= NBIG * f) {
    const int per = up((hi - lo + NBIG - 1) / NBIG);
    if (link == 2) cuts.push_back(0);
    for (int c = lo; c < hi; c += per) cuts.push_back(c);
    if (link == 1) cuts.push_back(hi);
  } else {
    const int per = up((len + NS - 1) / NS);
    for (int c = 0; c < len; c += per) cuts.push_back(c);
  }
  cuts.push_back(len);
  cudaStream_t ms = cur_stream(), ps = g_pipe_stream, cs = g_copy_stream;
  // the second stream (and the copy stream) start after everything already queued on the
  // library stream
  if (cudaEventRecord(g_pipe_ev[kMaxSlabs], ms) != cudaSuccess ||
      cudaStreamWaitEvent(ps, g_pipe_ev[kMaxSlabs], 0) != cudaSuccess)
    return E_CUDA;
  if ((host_in || host_out) && cudaStreamWaitEvent(cs, g_pipe_ev[kMaxSlabs], 0) != cudaSuccess) return E_CUDA;
  ExecCtx pc{ps, nullptr, false, nullptr};
  const ExecCtx *prev = t_ctx;
  // stage a on the library stream and b on the priority stream, or the other way round when a
  // is the link stage
  const ExecCtx *ca = link == 1 ? &pc : prev, *cb = link == 1 ? prev : &pc;
  cudaStream_t sa = link == 1 ? ps : ms, sb = link == 1 ? ms : ps;
  // FP64: the link stage's CTAs take their tiles from a counter per slab, zeroed ahead of its
  // slabs on its own stream, so that the CTAs of a slab finish within about one tile of each
  // other (512^3 round trip 12.61 against 12.67 ms with a fixed grid stride; FP32, whose tiles
  // are shorter, 6.02 against 5.95 ms, keeps the grid stride)
  int *ctrs = (link && link_ctas > 0 && P->prec == 8 && tile_ctr_on()) ? tile_counters(g_tabs) : nullptr;
  if (ctrs && cudaMemsetAsync(ctrs, 0, sizeof(int) * kTileCounters, ps) != cudaSuccess) {
    cudaGetLastError();
    ctrs = nullptr;
  }
  int rc = E_OK;
  for (int k = 0; k + 1 < (int)cuts.size() && rc == E_OK; k++) {
    const int c = cuts[k];
    SlabBox box{sd, c, cuts[k + 1] - c};
    if (host_in) {
      if (cudaMemcpyAsync(static_cast<unsigned char *>(const_cast<void *>(src)) + (size_t)c * u[0],
                          static_cast<const unsigned char *>(host_in) + (size_t)c * u[0], (size_t)box.m * u[0],
                          cudaMemcpyHostToDevice, cs) != cudaSuccess ||
          cudaEventRecord(g_slab_ev[k], cs) != cudaSuccess || cudaStreamWaitEvent(sa, g_slab_ev[k], 0) != cudaSuccess) {
        rc = E_CUDA;
        break;
      }
    }
    box.ctas = link == 1 ? link_ctas : 0;
    box.ctr = (link == 1 && ctrs) ? ctrs + k : nullptr;
    t_ctx = ca;
    rc = run_stage(P, a, src, mid, da, nullptr, nullptr, -1, lka, &box);
    t_ctx = prev;
    if (rc != E_OK) break;
    if (cudaEventRecord(g_pipe_ev[k], sa) != cudaSuccess || cudaStreamWaitEvent(sb, g_pipe_ev[k], 0) != cudaSuccess) {
      rc = E_CUDA;
      break;
    }
    box.ctas = link == 2 ? link_ctas : 0;
    box.ctr = (link == 2 && ctrs) ? ctrs + k : nullptr;
    t_ctx = cb;
    rc = run_stage(P, b, mid, dst, db, nullptr, nullptr, -1, lkb, &box);
    t_ctx = prev;
    if (rc == E_OK && host_out) {
      if (cudaEventRecord(g_slab_ev[kMaxSlabs + k], sb) != cudaSuccess ||
          cudaStreamWaitEvent(cs, g_slab_ev[kMaxSlabs + k], 0) != cudaSuccess ||
          cudaMemcpyAsync(static_cast<unsigned char *>(host_out) + (size_t)c * u[3],
                          static_cast<const unsigned char *>(dst) + (size_t)c * u[3], (size_t)box.m * u[3],
                          cudaMemcpyDeviceToHost, cs) != cudaSuccess)
        rc = E_CUDA;
    }
  }
  if (host_out) {  // the library stream continues after the last copy
    if (cudaEventRecord(g_slab_ev[2 * kMaxSlabs], cs) != cudaSuccess ||
        cudaStreamWaitEvent(ms, g_slab_ev[2 * kMaxSlabs], 0) != cudaSuccess)
      return E_CUDA;
  }
  // the library stream continues after the second stream's last slab (also after a failure)
  if (cudaEventRecord(g_pipe_ev[kMaxSlabs], ps) != cudaSuccess ||
      cudaStreamWaitEvent(ms, g_pipe_ev[kMaxSlabs], 0) != cudaSuccess)
    return E_CUDA;
  return rc;
}

// Whether stage s of the plan runs on a kernel whose grid can be capped (StageDesc::max_ctas).
static bool link_cap_ok(const Plan *P, int s, const void *src, void *dst, int idir) {
  const Stage &st = P->ex[s];
  if (g_types[st.type].kind == K_EMPTY) return false;
  StageDesc d;
  fill_stage_desc(P, st, idir >= 0 && st.dim == idir, d);
  return stage_cap_ok(d, src, dst, P->prec == 8 ? arith_mode() : AR_NATIVE, g_tabs);
}

static int exec_plan(Plan *P, const void *in, void *out, int idir, int OW, cudaEvent_t *stage_ev = nullptr) {
  if (g_autotune && !in_capture() && (P->tune.empty() || (P->prec == 8 && P->tuned_arith != arith_mode()))) {
    if (!ensure_device()) return t_err;
    int rc = autotune_plan(P);
    if (rc != E_OK) return rc;
  }
  if (!ensure_device()) return t_err;
  if (!in || !out) {
    set_err(E_BAD_ARG, "null data pointer");
    return E_BAD_ARG;
  }
  (void)OW;  // the GPU path never modifies `in` unless in == out
  const size_t in_bytes = (size_t)elems(P->g1) * P->dt1 * P->prec;
  const size_t out_bytes = (size_t)elems(P->g2) * P->dt2 * P->prec;
  const bool din_dev = is_device_ptr(in), dout_dev = is_device_ptr(out);
  const void *din = in;
  void *dout = out;
  Buffers &B = (t_ctx && t_ctx->buf) ? *t_ctx->buf : P->buf;
  if (t_ctx && (!din_dev || !dout_dev)) {
    set_err(E_BAD_ARG, "batched execution takes device pointers only");
    return E_BAD_ARG;
  }
  // Page-locked host arrays are read by the first stage and written by the last stage directly
  // over NVLink-C2C, with no staging copy; pageable host arrays are staged through HBM.
  void *in_mapped = (din_dev || !(host_direct_mode() & 1)) ? nullptr : mapped_host_ptr(in);
  void *out_mapped = (dout_dev || !(host_direct_mode() & 2)) ? nullptr : mapped_host_ptr(out);
  const bool in_direct = in_mapped && in != out;
  if (in_direct) din = in_mapped;
  const bool out_direct = out_mapped && in != out;
  if (out_direct) dout = out_mapped;
  const int n = (int)P->ex.size();
  // Host staging overlapped with the first / last stage: the copy of slab c runs on the copy
  // stream while the stage works on slab c-1 (slabs along a dim that is the slowest of the
  // stage's input and output layouts, so each slab is contiguous on both sides).
  const bool stage_host_in = !din_dev && !in_direct, stage_host_out = !dout_dev && !out_direct;
  // (only for fields of 32 MB and more: below that, one copy costs less than the extra launches)
  const size_t kSlabMin = 32u << 20;
  const int sd_in = (stage_host_in && in_bytes >= kSlabMin && n >= 2 && !stage_ev && !g_timers_on)
                        ? slab_dim(P->ex[0]) : -1;
  const int sd_out = (stage_host_out && out_bytes >= kSlabMin && n >= 2 && !stage_ev && !g_timers_on && in != out)
                         ? slab_dim(P->ex[n - 1]) : -1;
  // Staged host arrays: the first stage and the next one run slab by slab, each slab's host copy
  // on the copy stream just before the first stage's slab and the second stage's slab right
  // after it on a second stream; likewise the last two stages with the copies back (the slab dim
  // the slowest of the staged layout, so each slab is one copy).  Not for host arrays read or
  // written directly by the kernels: there the SMs themselves move the data over the link and
  // a concurrent stage only takes SM time from them (measured no gain, 13.69 vs 13.66 ms).
  // Host arrays read or written directly: with a grid cap on the link stage (link_ctas), the
  // neighbour stage runs slab by slab on the SMs the link stage leaves free.
  const bool can_pipe = !stage_ev && !g_timers_on && !t_ctx && n >= 3 && pipeline_host_stages();
  int pipe_in = -1, pipe_out = -1;
  if (can_pipe && stage_host_in && in_bytes >= kSlabMin) {
    pipe_in = pair_slab_dim(P->ex[0], P->ex[1]);
    if (pipe_in >= 0 && P->ex[0].g1.mo[pipe_in] != 2) pipe_in = -1;
  }
  if (can_pipe && stage_host_out && out_bytes >= kSlabMin && (pipe_in < 0 || n >= 4) && in != out) {
    pipe_out = pair_slab_dim(P->ex[n - 2], P->ex[n - 1]);
    if (pipe_out >= 0 && P->ex[n - 1].g2.mo[pipe_out] != 2) pipe_out = -1;
  }
  const bool pipe_in_staged = pipe_in >= 0 && stage_host_in, pipe_out_staged = pipe_out >= 0 && stage_host_out;
  if (stage_host_in) {
    if (!ensure_buf(&B.stage_in, &B.stage_in_bytes, in_bytes)) return E_CUDA;
    if (sd_in < 0 && !pipe_in_staged) {
      TimerScope ts(4);
      if (cudaMemcpyAsync(B.stage_in, in, in_bytes, cudaMemcpyHostToDevice, cur_stream()) != cudaSuccess) {
        set_err(E_CUDA, "host-to-device copy failed");
        return E_CUDA;
      }
    }
    din = B.stage_in;
  }
  if (stage_host_out) {
    if (!ensure_buf(&B.stage_out, &B.stage_out_bytes, out_bytes)) return E_CUDA;
    dout = B.stage_out;
  }
  // buffer assignment: consecutive stages never share a buffer and stage 0 never writes `in`
  size_t need = 0;
  for (int s = 0; s < n - 1; s++) need = std::max(need, stage_out_bytes(P, P->ex[s]));
  std::vector<void *> dst(n, nullptr);
  dst[n - 1] = dout;
  int nscratch_used = 0;
  for (int s = n - 2; s >= 0; s--) {
    size_t bytes = stage_out_bytes(P, P->ex[s]);
    void *cand = nullptr;
    // (a staged output pipelined with the stage before the last: the slabs of stage n-2 read
    // dst[n-3] while the last stage writes the output buffer, so they must differ)
    if (!out_direct && dout != dst[s + 1] && bytes <= out_bytes && !(s == 0 && dout == din) && dout != din &&
        !(pipe_out_staged && s == n - 3))
      cand = dout;
    if (!cand) {
      int k = (dst[s + 1] == B.scratch[0] && B.scratch[0]) ? 1 : 0;
      if (need > B.scratch_bytes || !B.scratch[k]) {
        if (in_capture() || !B.owned) {  // a graph must not record an allocation
          set_err(E_PLAN, "scratch set too small for a captured plan (%zu bytes needed)", need);
          return E_PLAN;
        }
        // (re)allocate both scratch slots at the common size on first use
        for (int i = 0; i < 2; i++)
          if (B.scratch[i] && B.scratch_bytes < need) {
            cudaFree(B.scratch[i]);
            B.scratch[i] = nullptr;
          }
        size_t have = B.scratch_bytes < need ? 0 : B.scratch_bytes;
        if (!B.scratch[k]) {
          if (cudaMalloc(&B.scratch[k], need) != cudaSuccess) {
            cudaGetLastError();
            B.scratch[k] = nullptr;
            set_err(E_CUDA, "cudaMalloc of %zu bytes (stage scratch) failed", need);
            return E_CUDA;
          }
        }
        B.scratch_bytes = std::max(have, need);
      }
      cand = B.scratch[k];
      nscratch_used++;
    }
    dst[s] = cand;
  }
  // Host arrays read or written directly: the link stage capped at lc persistent CTAs (when its
  // kernel has that form) and its neighbour stage beside it, slab by slab.
  const int lc = can_pipe && (in_direct || out_direct) ? link_ctas(P->prec) : 0;
  if (lc > 0 && in_direct && pipe_in < 0 && in_bytes >= kSlabMin && link_cap_ok(P, 0, din, dst[0], idir))
    pipe_in = pair_slab_dim(P->ex[0], P->ex[1]);
  if (lc > 0 && out_direct && pipe_out < 0 && out_bytes >= kSlabMin && (pipe_in < 0 || n >= 4) &&
      link_cap_ok(P, n - 1, dst[n - 2], dout, idir))
    pipe_out = pair_slab_dim(P->ex[n - 2], P->ex[n - 1]);
  // float-float links between consecutive specialised float-float stages (not for recorded or
  // caller-owned scratch sets, slab-pipelined host stages or in-place single-stage calls)
  std::vector<FFLink> ffl(n);
  if (ff_intermediates() && n >= 2 && !t_ctx && B.owned && P->prec == 8 && arith_mode() == AR_DF) {
    std::vector<char> cin(n, 0), cout_(n, 0);
    const void *qs = din;
    for (int s = 0; s < n; s++) {
      const Stage &st = P->ex[s];
      const bool deriv = idir >= 0 && st.dim == idir && g_types[st.type].kind != K_EMPTY;
      bool ci = false, co = false;
      if (dst[s] != qs) stage_ff_capable(P, st, qs, dst[s], deriv, &ci, &co);
      cin[s] = ci;
      cout_[s] = co;
      qs = dst[s];
    }
    for (int s = 0; s + 1 < n; s++) {
      if (!cout_[s] || !cin[s + 1]) continue;
      const Stage &st = P->ex[s];
      const int k = s & 1;
      const size_t bytes = (size_t)(elems(st.g2) / st.g2.gdims[st.dim]) * sizeof(int);
      if (bytes > B.side_bytes[k] || !B.side[k]) {
        // no allocation inside a stream capture: this boundary stays IEEE
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (in_capture() || cudaStreamIsCapturing(cur_stream(), &cs) != cudaSuccess ||
            cs != cudaStreamCaptureStatusNone) {
          cudaGetLastError();
          continue;
        }
        if (!ensure_buf(&B.side[k], &B.side_bytes[k], bytes)) return E_CUDA;
      }
      long long m[3];
      ff_multipliers(st.g2, st.dim, P->ex[s + 1].dim, m);
      ffl[s].ffout = 1;
      ffl[s].sout = static_cast<int *>(B.side[k]);
      ffl[s + 1].ffin = 1;
      ffl[s + 1].sin = static_cast<const int *>(B.side[k]);
      for (int i = 0; i < 3; i++) {
        ffl[s].mo[i] = m[i];
        ffl[s + 1].mi[i] = m[i];
      }
    }
  }
  const void *src = din;
  int rc = E_OK;
  for (int s = 0; s < n && rc == E_OK; s++) {
    const Stage &st = P->ex[s];
    bool deriv = idir >= 0 && st.dim == idir && g_types[st.type].kind != K_EMPTY;
    void *d = dst[s];
    if (stage_ev) cudaEventRecord(stage_ev[s], cur_stream());
    const FFLink *lk = (ffl[s].ffin || ffl[s].ffout) ? &ffl[s] : nullptr;
    if ((s == 0 && pipe_in >= 0) || (s == n - 2 && pipe_out >= 0)) {  // this stage and the next, pipelined
      const FFLink *lk2 = (ffl[s + 1].ffin || ffl[s + 1].ffout) ? &ffl[s + 1] : nullptr;
      const bool first = s == 0 && pipe_in >= 0;
      const int link = first ? (pipe_in_staged ? 0 : 1) : (pipe_out_staged ? 0 : 2);
      rc = run_pair_slabs(P, s, src, d, dst[s + 1], idir, lk, lk2, first ? pipe_in : pipe_out,
                          (first && pipe_in_staged) ? in : nullptr, (!first && pipe_out_staged) ? out : nullptr,
                          link, lc);
      src = dst[s + 1];
      s++;
      continue;
    } else if (s == 0 && sd_in >= 0) {
      rc = run_stage_slabs(P, st, sd_in, in, din, d, deriv, 0, lk);
    } else if (s == n - 1 && sd_out >= 0) {
      rc = run_stage_slabs(P, st, sd_out, out, src, d, deriv, 1, lk);
    } else if (d == src && t_ctx && t_ctx->rec) {
      set_err(E_UNSUPPORTED, "an in-place single-stage plan cannot be recorded for a grouped launch");
      return E_UNSUPPORTED;
    } else if (d == src) {  // single-stage in-place call: go through scratch, then copy back
      size_t bytes = stage_out_bytes(P, st);
      if ((in_capture() || !B.owned) && (bytes > B.scratch_bytes || !B.scratch[0])) {
        set_err(E_PLAN, "scratch set too small for an in-place stage (%zu bytes needed)", bytes);
        return E_PLAN;
      }
      if (!ensure_buf(&B.scratch[0], &B.scratch_bytes, std::max(bytes, B.scratch_bytes))) return E_CUDA;
      rc = run_stage(P, st, src, B.scratch[0], deriv);
      if (rc == E_OK && cudaMemcpyAsync(d, B.scratch[0], bytes, cudaMemcpyDeviceToDevice, cur_stream()) != cudaSuccess)
        rc = E_CUDA;
    } else {
      rc = run_stage(P, st, src, d, deriv, nullptr, nullptr, -1, lk);
    }
    src = d;
  }
  if (stage_ev) cudaEventRecord(stage_ev[n], cur_stream());
  if (rc != E_OK) return rc;
  if (stage_host_out && sd_out < 0 && !pipe_out_staged) {
    TimerScope ts(5);
    if (cudaMemcpyAsync(out, dout, out_bytes, cudaMemcpyDeviceToHost, cur_stream()) != cudaSuccess) {
      set_err(E_CUDA, "device-to-host copy failed");
      return E_CUDA;
    }
  }
  if (!t_ctx && (g_sync || !din_dev || !dout_dev)) {
    cudaError_t e = cudaStreamSynchronize(cur_stream());
    if (e != cudaSuccess) {
      set_err(E_CUDA, "stream synchronize failed: %s", cudaGetErrorString(e));
      return E_CUDA;
    }
  }
  return E_OK;
}

static Plan *get_plan(std::vector<Plan *> &v, int h) {
  std::lock_guard<std::mutex> g(g_mu);
  if (h < 0 || h >= (int)v.size() || !v[h]) return nullptr;
  return v[h];
}

static int store_plan(std::vector<Plan *> &v, Plan *P) {
  std::lock_guard<std::mutex> g(g_mu);
  v.push_back(P);
  return (int)v.size() - 1;
}

// Runs a 3D plan entirely in caller-provided device memory: `scratch0` / `scratch1` hold the
// intermediate fields (each `scratch_bytes` long) and `tw_dev` (tw_bytes) the twiddle tables,
// which are generated into `tw_host` and copied in stream order.  Makes no device allocation.
int exec_plan_given_memory(int plan, const void *in, void *out, int idir, void *scratch0, void *scratch1,
                           size_t scratch_bytes, void *tw_dev, size_t tw_bytes, void *tw_host) {
  // The tables are staged through the host array tw_host, which the next call overwrites: a
  // captured graph would copy whatever it holds at replay time, so capture is refused.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(cur_stream(), &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    set_err(E_UNSUPPORTED, "this entry point stages its tables through host memory and cannot run on a capturing stream");
    return E_UNSUPPORTED;
  }
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 3D plan handle %d", plan);
    return E_BAD_ARG;
  }
  if (idir > 2) {
    set_err(E_BAD_ARG, "derivative direction %d out of range", idir);
    return E_BAD_ARG;
  }
  if (!in || !out || !is_device_ptr(in) || !is_device_ptr(out)) {
    set_err(E_BAD_ARG, "this entry point takes device pointers only (host data would need staging buffers)");
    return E_BAD_ARG;
  }
  const int n = (int)P->ex.size();
  const size_t out_bytes = (size_t)elems(P->g2) * P->dt2 * P->prec;
  // buffer assignment as in exec_plan, with the two given scratch buffers
  void *dst[8];
  dst[n - 1] = out;
  for (int s = n - 2; s >= 0; s--) {
    size_t bytes = stage_out_bytes(P, P->ex[s]);
    if (out != dst[s + 1] && out != in && bytes <= out_bytes) dst[s] = out;
    else dst[s] = (dst[s + 1] == scratch0) ? scratch1 : scratch0;
    if ((dst[s] == scratch0 || dst[s] == scratch1) && bytes > scratch_bytes) {
      set_err(E_TOO_LARGE, "intermediate field of %zu bytes exceeds the %zu-byte static scratch buffer", bytes,
              scratch_bytes);
      return E_TOO_LARGE;
    }
  }
  if (n == 1 && in == out) {
    set_err(E_BAD_ARG, "single-stage in-place transform needs an extra buffer; pass in != out");
    return E_BAD_ARG;
  }
  // twiddle tables of every stage, packed into the given region.  Each stage's needs are queried
  // with the derivative flag and the buffers it will run with, so that the query and the launch
  // choose the same kernel (and table format).  A tuned engine that needs cached tables (Bluestein,
  // the specialised DCT/DST II-IV kernel) falls back to the heuristic choice.
  const void *tw[8] = {nullptr}, *aux[8] = {nullptr};
  int eng[8];
  size_t off = 0;
  unsigned char *host = static_cast<unsigned char *>(tw_host);
  const void *qsrc = in;
  for (int s = 0; s < n; s++) {
    const Stage &st = P->ex[s];
    eng[s] = -1;
    const void *ssrc = qsrc;
    qsrc = dst[s];
    if (g_types[st.type].kind == K_EMPTY) continue;
    const bool deriv = idir >= 0 && st.dim == idir;
    StageDesc d;
    fill_stage_desc(P, st, deriv, d);
    TableNeed need{0, 0, 0, 0};
    const int arith = P->prec == 8 ? arith_mode() : AR_NATIVE;
    int rc = launch_stage(d, ssrc, dst[s], arith, cur_stream(), nullptr, nullptr, nullptr, nullptr, &need);
    if (rc == E_UNSUPPORTED && d.engine != 0) {
      d.engine = 0;
      eng[s] = 0;
      rc = launch_stage(d, ssrc, dst[s], arith, cur_stream(), nullptr, nullptr, nullptr, nullptr, &need);
    }
    if (rc != E_OK) {
      set_err(rc, "stage %d cannot run with caller-supplied tables (length %d unsupported on this path)", s,
              st.g1.gdims[st.dim]);
      return rc;
    }
    const size_t b1 = table_bytes(need.tabN, need.fmt);
    const size_t b2 = need.auxN ? (need.aux_pass ? pass_table_bytes(need.auxN, need.fmt) : table_bytes(need.auxN, need.fmt)) : 0;
    const size_t a1 = (b1 + 255) & ~(size_t)255, a2 = (b2 + 255) & ~(size_t)255;
    if (off + a1 + a2 > tw_bytes) {  // both tables, each starting on a 256-byte boundary
      set_err(E_TOO_LARGE, "twiddle tables exceed the %zu-byte static table region", tw_bytes);
      return E_TOO_LARGE;
    }
    fill_table(need.tabN, need.fmt, host + off);
    tw[s] = static_cast<unsigned char *>(tw_dev) + off;
    off += a1;
    if (b2) {
      if (need.aux_pass) fill_pass_table(need.auxN, need.fmt, host + off);
      else fill_table(need.auxN, need.fmt, host + off);
      aux[s] = static_cast<unsigned char *>(tw_dev) + off;
      off += a2;
    }
  }
  if (off && cudaMemcpyAsync(tw_dev, tw_host, off, cudaMemcpyHostToDevice, cur_stream()) != cudaSuccess) {
    set_err(E_CUDA, "twiddle upload failed");
    return E_CUDA;
  }
  const void *src = in;
  for (int s = 0; s < n; s++) {
    const Stage &st = P->ex[s];
    bool deriv = idir >= 0 && st.dim == idir && g_types[st.type].kind != K_EMPTY;
    int rc = run_stage(P, st, src, dst[s], deriv, tw[s], aux[s], eng[s]);
    if (rc != E_OK) return rc;
    src = dst[s];
  }
  if (g_sync) {
    cudaError_t e = cudaStreamSynchronize(cur_stream());
    if (e != cudaSuccess) {
      set_err(E_CUDA, "stream synchronize failed: %s", cudaGetErrorString(e));
      return E_CUDA;
    }
  }
  return E_OK;
}

void record_error(int code, const char *msg) { set_err(code, "%s", msg); }

// ---- executor interface for the batch and serving runtimes (runtime.h) ----
void *scratch_set_create() { return new Buffers(); }

void scratch_set_destroy(void *b) {
  if (!b) return;
  Buffers *B = static_cast<Buffers *>(b);
  B->release();
  delete B;
}

size_t scratch_set_bytes(const void *b) { return b ? static_cast<const Buffers *>(b)->scratch_bytes : 0; }

void *scratch_set_wrap(void *s0, void *s1, size_t bytes) {
  Buffers *B = new Buffers();
  B->scratch[0] = s0;
  B->scratch[1] = s1;
  B->scratch_bytes = bytes;
  B->owned = false;
  return B;
}

int scratch_set_reserve(void *b, size_t bytes) {
  Buffers *B = static_cast<Buffers *>(b);
  if (bytes <= B->scratch_bytes && B->scratch[0] && B->scratch[1]) return E_OK;
  for (int i = 0; i < 2; i++) {
    if (B->scratch[i]) cudaFree(B->scratch[i]);
    B->scratch[i] = nullptr;
  }
  B->scratch_bytes = 0;
  for (int i = 0; i < 2; i++) {
    if (cudaMalloc(&B->scratch[i], bytes) != cudaSuccess) {
      cudaGetLastError();
      B->release();
      set_err(E_CUDA, "cudaMalloc of %zu bytes (scratch set) failed", bytes);
      return E_CUDA;
    }
  }
  B->scratch_bytes = bytes;
  return E_OK;
}

int plan3d_sizes(int plan, size_t *in_bytes, size_t *out_bytes, size_t *scratch_bytes, int *prec) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 3D plan handle %d", plan);
    return E_BAD_ARG;
  }
  size_t need = 0;
  for (size_t s = 0; s + 1 < P->ex.size(); s++) need = std::max(need, stage_out_bytes(P, P->ex[s]));
  if (in_bytes) *in_bytes = (size_t)elems(P->g1) * P->dt1 * P->prec;
  if (out_bytes) *out_bytes = (size_t)elems(P->g2) * P->dt2 * P->prec;
  if (scratch_bytes) *scratch_bytes = need;
  if (prec) *prec = P->prec;
  return E_OK;
}

int exec_plan_on(int plan, const void *in, void *out, int idir, cudaStream_t st, void *scratch_set, bool capturing) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 3D plan handle %d", plan);
    return E_BAD_ARG;
  }
  if (idir > 2) {
    set_err(E_BAD_ARG, "derivative direction %d out of range", idir);
    return E_BAD_ARG;
  }
  ExecCtx ctx{st, static_cast<Buffers *>(scratch_set), capturing, nullptr};
  const ExecCtx *prev = t_ctx;
  t_ctx = &ctx;
  int rc = exec_plan(P, in, out, idir, 0);
  t_ctx = prev;
  return rc;
}

int record_plan(int plan, const void *in, void *out, int idir, void *scratch_set, std::vector<StageLaunch> *rec) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 3D plan handle %d", plan);
    return E_BAD_ARG;
  }
  ExecCtx ctx{g_stream, static_cast<Buffers *>(scratch_set), false, rec};
  const ExecCtx *prev = t_ctx;
  t_ctx = &ctx;
  int rc = exec_plan(P, in, out, idir, 0);
  t_ctx = prev;
  return rc;
}

DeviceTables *device_tables() { return g_tabs; }

bool device_ready() { return ensure_device(); }
cudaStream_t library_stream() { return g_stream; }
bool library_sync() { return g_sync != 0; }
int current_arith() { return arith_mode(); }
void add_kernel_count(long long n) { g_kcount += n; }
long long kernel_count_now() { return g_kcount.load(); }

static void ensure_setup() {
  if (!g_setup_done) {
    build_registry();
    assign_globals();
    g_setup_done = true;
  }
}

}  // namespace p3d

using namespace p3d;

// ==========================================================================================
// GB300 extension C ABI (p3dfft_gb300.h)
extern "C" {

int p3dfft_last_error(void) { return t_err; }
const char *p3dfft_last_error_string(void) { return t_msg; }
void p3dfft_clear_error(void) {
  t_err = E_OK;
  snprintf(t_msg, sizeof(t_msg), "no error");
}
void p3dfft_gb300_set_stream(void *s) { g_stream = (cudaStream_t)s; }
void p3dfft_gb300_set_sync(int s) { g_sync = s ? 1 : 0; }
void p3dfft_gb300_set_host_pipeline(int on) { g_host_pipe = on ? 1 : 0; }
void p3dfft_gb300_set_link_ctas(int n) { g_link_ctas = n < 0 ? -1 : n; }
void p3dfft_gb300_set_pageable_direct(int on) { g_pageable_direct = on ? 1 : 0; }
int p3dfft_gb300_get_pageable_direct(void) {
  if (!ensure_device()) return 0;
  return pageable_direct() ? 1 : (pageable_access_ok() ? 0 : -1);
}
int p3dfft_gb300_get_link_ctas(void) { return link_ctas_set(); }
int p3dfft_gb300_get_host_pipeline(void) { return pipeline_host_stages() ? 1 : 0; }
void p3dfft_gb300_set_host_direct(int on) { g_host_direct = on == 1 ? 3 : (on == 2 ? 1 : (on == 3 ? 2 : 0)); }
void p3dfft_gb300_set_fp64_arith(int m) { g_arith = m ? AR_DF : AR_NATIVE; }
void p3dfft_gb300_set_reference_compat(int on) { g_ref_compat = on ? 1 : 0; }
void p3dfft_gb300_set_ff_intermediates(int on) { g_ff_inter = on ? 1 : 0; }
void p3dfft_gb300_set_fp32_split_twiddles(int on) { set_fp32_split_twiddles(on != 0); }
int p3dfft_gb300_get_fp32_split_twiddles(void) { return fp32_split_twiddles() ? 1 : 0; }
void p3dfft_gb300_set_fp32_tma(int on) { set_fp32_tma(on != 0); }
int p3dfft_gb300_get_fp32_tma(void) { return fp32_tma() ? 1 : 0; }
int p3dfft_gb300_device_status(int clear) {
  if (!ensure_device()) return -1;
  return device_status(g_tabs, clear != 0);
}
void p3dfft_gb300_inject_tma_stall(void) { inject_tma_stall(); }
long long p3dfft_gb300_tma_launch_count(void) { return tma_launches(); }
int p3dfft_gb300_get_ff_intermediates(void) { return ff_intermediates() ? 1 : 0; }
int p3dfft_gb300_get_reference_compat(void) { return ref_compat(); }
int p3dfft_gb300_get_fp64_arith(void) { return arith_mode(); }
const char *p3dfft_gb300_version(void) { return "p3dfft-gb300 0.1 (sm_103a)"; }

int p3dfft_gb300_plan3d(const int types[3], const int gdims1[3], const int mo1[3], int dcs1, const int gdims2[3],
                        const int mo2[3], int dcs2) {
  ensure_setup();
  GridDesc g1{{gdims1[0], gdims1[1], gdims1[2]}, {mo1[0], mo1[1], mo1[2]}, dcs1};
  GridDesc g2{{gdims2[0], gdims2[1], gdims2[2]}, {mo2[0], mo2[1], mo2[2]}, dcs2};
  Plan *P = make_plan3(types, g1, g2);
  if (!P) return -1;
  return store_plan(g_plans3, P);
}

int p3dfft_gb300_exec3d(int plan, const void *in, void *out, int idir, int OW) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 3D plan handle %d", plan);
    return E_BAD_ARG;
  }
  if (idir > 2) {
    set_err(E_BAD_ARG, "derivative direction %d out of range", idir);
    return E_BAD_ARG;
  }
  return exec_plan(P, in, out, idir, OW);
}

// ---- autotuner ----
void p3dfft_gb300_set_autotune(int on) { g_autotune = on != 0; }

static Plan *plan_of(int plan, int is1d) { return get_plan(is1d ? g_plans1 : g_plans3, plan); }

int p3dfft_gb300_autotune(int plan, int is1d) {
  Plan *P = plan_of(plan, is1d);
  if (!P) {
    set_err(E_BAD_ARG, "invalid plan handle %d", plan);
    return E_BAD_ARG;
  }
  return autotune_plan(P);
}

int p3dfft_gb300_plan_tuning(int plan, int is1d, int *engine, int *talt, double *ms, int max_stages) {
  Plan *P = plan_of(plan, is1d);
  if (!P) return -1;
  const int n = (int)P->ex.size();
  for (int s = 0; s < n && s < max_stages; s++) {
    const bool t = P->tune.size() == P->ex.size();
    if (engine) engine[s] = t ? P->tune[s].engine : 0;
    if (talt) talt[s] = t ? P->tune[s].talt : 0;
    if (ms) ms[s] = t ? P->tune[s].ms : 0.0;
  }
  return n;
}

int p3dfft_gb300_plan_set_engine(int plan, int is1d, int stage, int engine, int talt) {
  Plan *P = plan_of(plan, is1d);
  if (!P || stage < 0 || stage >= (int)P->ex.size() || engine < 0 || engine > ENG_BLUESTEIN) {
    set_err(E_BAD_ARG, "invalid plan, stage or engine");
    return E_BAD_ARG;
  }
  if (P->tune.size() != P->ex.size()) P->tune.assign(P->ex.size(), StageTune());
  P->tune[stage].engine = engine;
  P->tune[stage].talt = talt ? 1 : 0;
  P->tuned_arith = arith_mode();
  return E_OK;
}

int p3dfft_gb300_tune_cache_save(const char *path) {
  FILE *f = path ? fopen(path, "w") : nullptr;
  if (!f) {
    set_err(E_BAD_ARG, "cannot write tuning cache %s", path ? path : "(null)");
    return E_BAD_ARG;
  }
  std::lock_guard<std::mutex> g(g_tmu);
  fprintf(f, "# p3dfft_gb300 tuning cache: stage key | engine talt ms\n");
  for (auto &kv : g_tune_cache) fprintf(f, "%s | %d %d %.9g\n", kv.first.c_str(), kv.second.engine, kv.second.talt, (double)kv.second.ms);
  fclose(f);
  return E_OK;
}

// returns the number of entries read, or -1
int p3dfft_gb300_tune_cache_load(const char *path) {
  FILE *f = path ? fopen(path, "r") : nullptr;
  if (!f) {
    set_err(E_BAD_ARG, "cannot read tuning cache %s", path ? path : "(null)");
    return -1;
  }
  char line[512];
  int n = 0;
  std::lock_guard<std::mutex> g(g_tmu);
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    char *bar = strchr(line, '|');
    if (!bar) continue;
    *bar = 0;
    std::string key(line);
    while (!key.empty() && key.back() == ' ') key.pop_back();
    StageTune t;
    if (sscanf(bar + 1, "%d %d %f", &t.engine, &t.talt, &t.ms) != 3 || t.engine < 0 || t.engine > ENG_BLUESTEIN) continue;
    g_tune_cache[key] = t;
    n++;
  }
  fclose(f);
  return n;
}

void p3dfft_gb300_tune_cache_clear(void) {
  std::lock_guard<std::mutex> g(g_tmu);
  g_tune_cache.clear();
}

int p3dfft_gb300_destroy3d(int plan) {
  std::lock_guard<std::mutex> g(g_mu);
  if (plan < 0 || plan >= (int)g_plans3.size() || !g_plans3[plan]) return E_BAD_ARG;
  g_plans3[plan]->buf.release();
  delete g_plans3[plan];
  g_plans3[plan] = nullptr;
  return E_OK;
}

int p3dfft_gb300_plan3d_types(int plan, int *dt1, int *dt2, int *prec) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) return E_BAD_ARG;
  *dt1 = P->dt1;
  *dt2 = P->dt2;
  *prec = P->prec;
  return E_OK;
}

static int stages_info(const std::vector<Stage> &v, int *info, int max_stages) {
  int n = (int)v.size();
  for (int s = 0; s < n && s < max_stages; s++) {
    const Stage &st = v[s];
    int *q = info + 16 * s;
    q[0] = st.type;
    q[1] = st.dim;
    for (int i = 0; i < 3; i++) {
      q[2 + i] = st.g1.gdims[i];
      q[5 + i] = st.g1.mo[i];
      q[9 + i] = st.g2.gdims[i];
      q[12 + i] = st.g2.mo[i];
    }
    q[8] = st.g1.dcs;
    q[15] = st.g2.dcs;
  }
  return n;
}

int p3dfft_gb300_plan3d_stages(int plan, int *info, int max_stages) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) return -1;
  return stages_info(P->st, info, max_stages);
}

int p3dfft_gb300_plan3d_exec_stages(int plan, int *info, int max_stages) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) return -1;
  return stages_info(P->ex, info, max_stages);
}

int p3dfft_gb300_plan1d(int type, const int gdims1[3], const int mo1[3], int dcs1, const int gdims2[3],
                        const int mo2[3], int dcs2, int dim) {
  ensure_setup();
  GridDesc g1{{gdims1[0], gdims1[1], gdims1[2]}, {mo1[0], mo1[1], mo1[2]}, dcs1};
  GridDesc g2{{gdims2[0], gdims2[1], gdims2[2]}, {mo2[0], mo2[1], mo2[2]}, dcs2};
  Plan *P = make_plan1(type, g1, g2, dim);
  if (!P) return -1;
  return store_plan(g_plans1, P);
}

int p3dfft_gb300_exec1d(int plan, const void *in, void *out, int OW) {
  Plan *P = get_plan(g_plans1, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 1D plan handle %d", plan);
    return E_BAD_ARG;
  }
  return exec_plan(P, in, out, -1, OW);
}

int p3dfft_gb300_destroy1d(int plan) {
  std::lock_guard<std::mutex> g(g_mu);
  if (plan < 0 || plan >= (int)g_plans1.size() || !g_plans1[plan]) return E_BAD_ARG;
  g_plans1[plan]->buf.release();
  delete g_plans1[plan];
  g_plans1[plan] = nullptr;
  return E_OK;
}

int p3dfft_gb300_compute_deriv(int prec, const void *in, void *out, const int gdims[3], const int mo[3], int dcs,
                               int idir) {
  ensure_setup();
  if (!ensure_device()) return t_err;
  GridDesc g{{gdims[0], gdims[1], gdims[2]}, {mo[0], mo[1], mo[2]}, dcs};
  if (!valid_grid(g) || idir < 0 || idir > 2 || (prec != 4 && prec != 8) || !in || !out) {
    set_err(E_BAD_ARG, "compute_deriv: invalid arguments");
    return E_BAD_ARG;
  }
  size_t bytes = (size_t)elems(g) * 2 * prec;
  long long s[3];
  strides(g, s);
  // g = (N-1)*2 along the conjugate-symmetric dim, else N (deriv.C:95-99)
  int gg = (dcs == idir) ? (gdims[idir] - 1) * 2 : gdims[idir];
  bool hin = !is_device_ptr(in), hout = !is_device_ptr(out);
  static thread_local Buffers B;
  const void *din = in;
  void *dout = out;
  if (hin) {
    if (!ensure_buf(&B.stage_in, &B.stage_in_bytes, bytes)) return E_CUDA;
    cudaMemcpyAsync(B.stage_in, in, bytes, cudaMemcpyHostToDevice, g_stream);
    din = B.stage_in;
  }
  if (hout) {
    if (!ensure_buf(&B.stage_out, &B.stage_out_bytes, bytes)) return E_CUDA;
    dout = B.stage_out;
  }
  int launched = 0;
  int rc = launch_deriv(prec, g.gdims, s, idir, gg, ref_compat(), din, dout, g_stream, &launched);
  g_kcount += launched;
  if (rc != E_OK) {
    set_err(rc, "compute_deriv launch failed");
    return rc;
  }
  if (hout) cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, g_stream);
  if (g_sync || hin || hout) {
    if (cudaStreamSynchronize(g_stream) != cudaSuccess) {
      set_err(E_CUDA, "compute_deriv: synchronize failed");
      return E_CUDA;
    }
  }
  return E_OK;
}

static cudaEvent_t g_events[64];
static bool g_events_made = false;

int p3dfft_gb300_event_record(int slot) {
  if (slot < 0 || slot >= 64 || !ensure_device()) return E_BAD_ARG;
  if (!g_events_made) {
    for (auto &e : g_events) cudaEventCreate(&e);
    g_events_made = true;
  }
  return cudaEventRecord(g_events[slot], g_stream) == cudaSuccess ? E_OK : E_CUDA;
}

double p3dfft_gb300_event_elapsed_ms(int a, int b) {
  if (!g_events_made || a < 0 || a >= 64 || b < 0 || b >= 64) return -1.0;
  if (cudaEventSynchronize(g_events[b]) != cudaSuccess) return -1.0;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, g_events[a], g_events[b]) != cudaSuccess) return -1.0;
  return (double)ms;
}

int p3dfft_gb300_profile_stages(int plan, const void *in, void *out, int idir, int reps, double *ms, int max_stages) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "invalid 3D plan handle %d", plan);
    return -1;
  }
  if (!ensure_device()) return -1;
  const int n = (int)P->ex.size();
  std::vector<cudaEvent_t> ev(n + 1);
  for (auto &e : ev) cudaEventCreate(&e);
  std::vector<double> acc(n, 0.0);
  // one untimed run first: twiddle tables, scratch fields and the lazy load of each kernel
  int rc = exec_plan(P, in, out, idir, 0);
  cudaStreamSynchronize(g_stream);
  for (int r = 0; r < reps && rc == E_OK; r++) {
    rc = exec_plan(P, in, out, idir, 0, ev.data());
    cudaEventSynchronize(ev[n]);
    for (int s = 0; s < n; s++) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[s], ev[s + 1]);
      acc[s] += t;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  for (int s = 0; s < n && s < max_stages; s++) ms[s] = reps > 0 ? acc[s] / reps : 0.0;
  return rc == E_OK ? n : -1;
}

int p3dfft_gb300_preload_kernels(void) {
  if (!ensure_device()) return t_err;
  const int rc = preload_kernels();
  if (rc != E_OK) set_err(rc, "kernel preload failed: %s", cudaGetErrorString(cudaGetLastError()));
  return rc;
}

long long p3dfft_gb300_kernel_count(void) { return g_kcount.load(); }
void p3dfft_gb300_reset_kernel_count(void) { g_kcount = 0; }
void p3dfft_gb300_enable_timers(int on) { g_timers_on = on != 0; }
double p3dfft_gb300_timer(int phase) { return (phase >= 0 && phase < 6) ? g_timer[phase] : 0.0; }
void p3dfft_gb300_reset_timers(void) {
  for (double &t : g_timer) t = 0;
}
void *p3dfft_gb300_device_alloc(long long bytes) {
  if (!ensure_device()) return nullptr;
  void *p = nullptr;
  if (cudaMalloc(&p, (size_t)bytes) != cudaSuccess) {
    cudaGetLastError();
    set_err(E_CUDA, "device allocation of %lld bytes failed", bytes);
    return nullptr;
  }
  return p;
}
void *p3dfft_gb300_host_alloc_pinned(long long bytes) {
  if (!ensure_device()) return nullptr;
  void *p = nullptr;
  if (cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) {
    cudaGetLastError();
    set_err(E_CUDA, "pinned host allocation of %lld bytes failed", bytes);
    return nullptr;
  }
  return p;
}
void p3dfft_gb300_host_free_pinned(void *p) {
  if (p) cudaFreeHost(p);
}
void p3dfft_gb300_device_free(void *p) {
  if (p) cudaFree(p);
}
int p3dfft_gb300_memcpy_h2d(void *dst, const void *src, long long bytes) {
  return cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyHostToDevice) == cudaSuccess ? E_OK : E_CUDA;
}
int p3dfft_gb300_memcpy_d2h(void *dst, const void *src, long long bytes) {
  return cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? E_OK : E_CUDA;
}
int p3dfft_gb300_synchronize(void) { return cudaStreamSynchronize(g_stream) == cudaSuccess ? E_OK : E_CUDA; }

int p3dfft_gb300_sm_count(void) {
  int dev = 0, n = 0;
  if (!ensure_device() || cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return n;
}

// ==========================================================================================
// Reference C ABI (Cwrap.h, build/wrap.C:85-571)

void p3dfft_setup() { ensure_setup(); }

void p3dfft_cleanup() {
  std::lock_guard<std::mutex> g(g_mu);
  for (auto *P : g_plans3)
    if (P) {
      P->buf.release();
      delete P;
    }
  for (auto *P : g_plans1)
    if (P) {
      P->buf.release();
      delete P;
    }
  g_plans3.clear();
  g_plans1.clear();
  g_types3d.clear();
  g_dgrids.clear();
  g_pgrids.clear();
  if (g_tabs) {
    tables_destroy(g_tabs);
    g_tabs = nullptr;
    g_device_ok = -1;
  }
}

Type3D p3dfft_init_3Dtype(int types[3]) {
  ensure_setup();
  Type3 t;
  for (int i = 0; i < 3; i++) t.types[i] = types[i];
  t.prec = (types[0] >= 0 && types[0] < 44) ? g_types[types[0]].prec : 0;
  std::lock_guard<std::mutex> g(g_mu);
  g_types3d.push_back(t);
  return (int)g_types3d.size() - 1;
}

int p3dfft_init_proc_grid(int pdims[3], MPI_Comm comm) {
  ensure_setup();
  if (pdims[0] * pdims[1] * pdims[2] != 1)
    set_err(E_UNSUPPORTED, "processor grid %d x %d x %d: only the 1x1x1 grid of one GPU is supported", pdims[0],
            pdims[1], pdims[2]);
  std::lock_guard<std::mutex> g(g_mu);
  g_pgrids.push_back(PGridRec{{pdims[0], pdims[1], pdims[2]}, comm, true});
  return (int)g_pgrids.size() - 1;
}

static int pgrid_nd(const int pd[3]) {
  int nd = 0;
  for (int i = 0; i < 3; i++)
    if (pd[i] > 1) nd++;
  return nd == 0 ? 1 : nd;
}

Grid *p3dfft_init_data_grid(int gdims[3], int dim_conj_sym, int pgrid_id, int dmap[3], int mem_order[3]) {
  ensure_setup();
  PGridRec pg;
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (pgrid_id < 0 || pgrid_id >= (int)g_pgrids.size()) {
      set_err(E_BAD_ARG, "p3dfft_init_data_grid: invalid processor grid %d", pgrid_id);
      return nullptr;
    }
    pg = g_pgrids[pgrid_id];
  }
  Grid *G = new Grid;
  memset(G, 0, sizeof(*G));
  G->numtasks = 1;
  G->taskid = 0;
  G->nd = pgrid_nd(pg.pdims);
  G->pgrid = pgrid_id;
  G->dim_conj_sym = dim_conj_sym;
  for (int i = 0; i < 3; i++) {
    G->Gdims[i] = gdims[i];
    G->Ldims[i] = gdims[i];
    G->MemOrder[i] = mem_order[i];
    G->Dmap[i] = dmap[i];
    G->ProcDims[i] = pg.pdims[i];
    G->grid_id[i] = 0;
    G->GlobStart[i] = 0;
  }
  G->mpi_comm_glob = pg.comm;
  return G;
}

void p3dfft_free_data_grid(Grid *gr) { delete gr; }

void p3dfft_free_proc_grid(int pgrid_id) {
  std::lock_guard<std::mutex> g(g_mu);
  if (pgrid_id >= 0 && pgrid_id < (int)g_pgrids.size()) g_pgrids[pgrid_id].live = false;
}

void p3dfft_inv_mo(int mo[3], int imo[3]) {
  for (int i = 0; i < 3; i++) imo[mo[i]] = i;
}

int find_grid(int gdims[3], int pgrid, int *dmap, int mem_order[3]) {
  std::lock_guard<std::mutex> g(g_mu);
  for (size_t i = 0; i < g_dgrids.size(); i++) {
    const DGridRec &r = g_dgrids[i];
    if (r.pgrid == pgrid && !memcmp(r.g.gdims, gdims, 3 * sizeof(int)) && !memcmp(r.dmap, dmap, 3 * sizeof(int)) &&
        !memcmp(r.g.mo, mem_order, 3 * sizeof(int)))
      return (int)i;
  }
  return -1;
}

Plan3D p3dfft_plan_3Dtrans(Grid *g1, Grid *g2, Type3D tp) {
  ensure_setup();
  Type3 t;
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (tp < 0 || tp >= (int)g_types3d.size()) {
      set_err(E_BAD_ARG, "p3dfft_plan_3Dtrans: invalid 3D type %d", tp);
      return -1;
    }
    t = g_types3d[tp];
  }
  if (!g1 || !g2) {
    set_err(E_BAD_ARG, "p3dfft_plan_3Dtrans: null grid");
    return -1;
  }
  return p3dfft_gb300_plan3d(t.types, g1->Gdims, g1->MemOrder, g1->dim_conj_sym, g2->Gdims, g2->MemOrder,
                             g2->dim_conj_sym);
}

int p3dfft_plan_1Dtrans(Grid *g1, Grid *g2, int type, int d) {
  if (!g1 || !g2) {
    set_err(E_BAD_ARG, "p3dfft_plan_1Dtrans: null grid");
    return -1;
  }
  return p3dfft_gb300_plan1d(type, g1->Gdims, g1->MemOrder, g1->dim_conj_sym, g2->Gdims, g2->MemOrder,
                             g2->dim_conj_sym, d);
}

static void exec3_checked(Plan3D plan, const void *in, void *out, int idir, int OW, int prec, const char *fn) {
  Plan *P = get_plan(g_plans3, plan);
  if (!P) {
    set_err(E_BAD_ARG, "%s: invalid plan %d", fn, plan);
    return;
  }
  if (P->prec != prec) {  // the reference calls MPI_Abort here (wrap.C:377-380)
    set_err(E_BAD_ARG, "%s: expecting %s precision data", fn, prec == 8 ? "double" : "single");
    return;
  }
  exec_plan(P, in, out, idir, OW);
}

void p3dfft_exec_3Dtrans_double(Plan3D plan, double *in, double *out, int OW) {
  exec3_checked(plan, in, out, -1, OW, 8, "p3dfft_exec_3Dtrans_double");
}
void p3dfft_exec_3Dtrans_single(Plan3D plan, float *in, float *out, int OW) {
  exec3_checked(plan, in, out, -1, OW, 4, "p3dfft_exec_3Dtrans_single");
}
void p3dfft_exec_3Dderiv_double(Plan3D plan, double *in, double *out, int idir, int OW) {
  exec3_checked(plan, in, out, idir, OW, 8, "p3dfft_exec_3Dderiv_double");
}
void p3dfft_exec_3Dderiv_single(Plan3D plan, float *in, float *out, int idir, int OW) {
  exec3_checked(plan, in, out, idir, OW, 4, "p3dfft_exec_3Dderiv_single");
}
void p3dfft_exec_1Dtrans_double(int plan, double *in, double *out, int OW) { p3dfft_gb300_exec1d(plan, in, out, OW); }
void p3dfft_exec_1Dtrans_single(int plan, float *in, float *out, int OW) { p3dfft_gb300_exec1d(plan, in, out, OW); }

void p3dfft_compute_deriv_single(float *in, float *out, Grid *g, int idir) {
  p3dfft_gb300_compute_deriv(4, in, out, g->Gdims, g->MemOrder, g->dim_conj_sym, idir);
}
void p3dfft_compute_deriv_double(double *in, double *out, Grid *g, int idir) {
  p3dfft_gb300_compute_deriv(8, in, out, g->Gdims, g->MemOrder, g->dim_conj_sym, idir);
}

// ---- Fortran glue (build/wrap.C:575-792): everything by reference, idir 1-based ----
void p3dfft_init_3Dtype_f(int *type, int types[3]) { *type = p3dfft_init_3Dtype(types); }

int p3dfft_init_proc_grid_f(int *pdims, int *mpicomm) { return p3dfft_init_proc_grid(pdims, (MPI_Comm)(*mpicomm)); }

void p3dfft_init_data_grid_f(int *mygrid, int *ldims, int *glob_start, int *gdims, int *dim_conj_sym, int *pgrid_id,
                             int *dmap, int *mem_order) {
  ensure_setup();
  int num = find_grid(gdims, *pgrid_id, dmap, mem_order);
  if (num < 0) {
    DGridRec r;
    for (int i = 0; i < 3; i++) {
      r.g.gdims[i] = gdims[i];
      r.g.mo[i] = mem_order[i];
      r.dmap[i] = dmap[i];
    }
    r.g.dcs = *dim_conj_sym;
    r.pgrid = *pgrid_id;
    std::lock_guard<std::mutex> g(g_mu);
    g_dgrids.push_back(r);
    num = (int)g_dgrids.size() - 1;
  }
  for (int i = 0; i < 3; i++) {
    ldims[i] = gdims[i];
    glob_start[i] = 0;
  }
  *mygrid = num;
}

static bool dgrid(int h, GridDesc *g) {
  std::lock_guard<std::mutex> l(g_mu);
  if (h < 0 || h >= (int)g_dgrids.size()) return false;
  *g = g_dgrids[h].g;
  return true;
}

void p3dfft_plan_3Dtrans_f(int *plan, int *Fgr1, int *Fgr2, Type3D *tp) {
  GridDesc a, b;
  Type3 t;
  *plan = -1;
  if (!dgrid(*Fgr1, &a) || !dgrid(*Fgr2, &b)) {
    set_err(E_BAD_ARG, "p3dfft_plan_3Dtrans_f: invalid grid handle");
    return;
  }
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (*tp < 0 || *tp >= (int)g_types3d.size()) {
      set_err(E_BAD_ARG, "p3dfft_plan_3Dtrans_f: invalid type");
      return;
    }
    t = g_types3d[*tp];
  }
  *plan = p3dfft_gb300_plan3d(t.types, a.gdims, a.mo, a.dcs, b.gdims, b.mo, b.dcs);
}

void p3dfft_plan_1Dtrans_f(int *plan, int *Fgr1, int *Fgr2, int *type, int *d) {
  GridDesc a, b;
  *plan = -1;
  if (!dgrid(*Fgr1, &a) || !dgrid(*Fgr2, &b)) {
    set_err(E_BAD_ARG, "p3dfft_plan_1Dtrans_f: invalid grid handle");
    return;
  }
  *plan = p3dfft_gb300_plan1d(*type, a.gdims, a.mo, a.dcs, b.gdims, b.mo, b.dcs, *d);
}

void p3dfft_exec_3Dtrans_double_f(Plan3D *plan, double *in, double *out, int *OW) {
  p3dfft_exec_3Dtrans_double(*plan, in, out, *OW);
}
void p3dfft_exec_3Dtrans_single_f(Plan3D *plan, float *in, float *out, int *OW) {
  p3dfft_exec_3Dtrans_single(*plan, in, out, *OW);
}
void p3dfft_exec_3Dderiv_double_f(Plan3D *plan, double *in, double *out, int *idir, int *OW) {
  p3dfft_exec_3Dderiv_double(*plan, in, out, *idir - 1, *OW);
}
void p3dfft_exec_3Dderiv_single_f(Plan3D *plan, float *in, float *out, int *idir, int *OW) {
  p3dfft_exec_3Dderiv_single(*plan, in, out, *idir - 1, *OW);
}
void p3dfft_exec_1Dtrans_double_f(int *plan, double *in, double *out, int *OW) {
  p3dfft_exec_1Dtrans_double(*plan, in, out, *OW);
}
void p3dfft_exec_1Dtrans_single_f(int *plan, float *in, float *out, int *OW) {
  p3dfft_exec_1Dtrans_single(*plan, in, out, *OW);
}
void p3dfft_compute_deriv_single_f(float *in, float *out, int *igrid, int *idir) {
  GridDesc g;
  if (!dgrid(*igrid, &g)) {
    set_err(E_BAD_ARG, "p3dfft_compute_deriv_single_f: invalid grid handle");
    return;
  }
  p3dfft_gb300_compute_deriv(4, in, out, g.gdims, g.mo, g.dcs, *idir - 1);
}
void p3dfft_compute_deriv_double_f(double *in, double *out, int *igrid, int *idir) {
  GridDesc g;
  if (!dgrid(*igrid, &g)) {
    set_err(E_BAD_ARG, "p3dfft_compute_deriv_double_f: invalid grid handle");
    return;
  }
  p3dfft_gb300_compute_deriv(8, in, out, g.gdims, g.mo, g.dcs, *idir - 1);
}

}  // extern "C"

// ==========================================================================================
// C++ API objects (reference include/p3dfft.h)
namespace p3dfft {

void setup() { p3dfft_setup(); }
void cleanup() { p3dfft_cleanup(); }
void inv_mo(int mo[3], int imo[3]) { p3dfft_inv_mo(mo, imo); }

// rel_change, build/exec.C:2270-2296: relative permutation between two inverse memory orders
void rel_change(int *imo1, int *imo2, int *m) {
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      if (imo1[j] == imo2[i]) m[j] = i;
}

ProcGrid::ProcGrid(int procdims[3], MPI_Comm mpi_comm_init) {
  p3d::ensure_setup();
  nd = 0;
  for (int i = 0; i < 3; i++) {
    ProcDims[i] = procdims[i];
    if (procdims[i] > 1) nd++;
    grid_id_cart[i] = 0;
    mpicomm[i] = mpi_comm_init;
  }
  if (nd == 0) nd = 1;
  taskid = 0;
  numtasks = 1;
  mpi_comm_glob = mpi_comm_init;
  mpi_comm_cart = mpi_comm_init;
  if (procdims[0] * procdims[1] * procdims[2] != 1)
    p3d::set_err(p3d::E_UNSUPPORTED, "ProcGrid %d x %d x %d: only the 1x1x1 grid of one GPU is supported",
                 procdims[0], procdims[1], procdims[2]);
}
ProcGrid::ProcGrid(const ProcGrid &r) {
  taskid = r.taskid;
  numtasks = r.numtasks;
  nd = r.nd;
  mpi_comm_glob = r.mpi_comm_glob;
  mpi_comm_cart = r.mpi_comm_cart;
  for (int i = 0; i < 3; i++) {
    ProcDims[i] = r.ProcDims[i];
    grid_id_cart[i] = r.grid_id_cart[i];
    mpicomm[i] = r.mpicomm[i];
  }
}
ProcGrid::~ProcGrid() {}
bool ProcGrid::operator==(const ProcGrid &P) const {
  if (nd != P.nd || taskid != P.taskid || numtasks != P.numtasks) return false;
  for (int i = 0; i < 3; i++)
    if (ProcDims[i] != P.ProcDims[i] || grid_id_cart[i] != P.grid_id_cart[i]) return false;
  return true;
}

// DataGrid ctor + InitPencil (init.C:1699-1729, 1806-1863) on one task: every dim is local
DataGrid::DataGrid(int *gdims_, int dim_conj_sym_, ProcGrid *pgrid, int *dmap, int *mem_order) {
  dim_conj_sym = dim_conj_sym_;
  Pgrid = pgrid;
  nd = pgrid ? pgrid->nd : 1;
  int ploc = 0, n = 0;
  for (int i = 0; i < 3; i++) {
    Gdims[i] = gdims_[i];
    Dmap[i] = dmap[i];
    Pdims[i] = pgrid ? pgrid->ProcDims[dmap[i]] : 1;
    MemOrder[i] = mem_order[i];
    grid_id[i] = 0;
    Ldims[i] = Gdims[i];
    GlobStart[i] = 0;
    D[i] = -1;
    L[i] = -1;
  }
  for (int k = 0; k < 3; k++) {
    if (Pdims[k] == 1) L[ploc++] = k;
    else D[n++] = k;
  }
  is_set = true;
}
DataGrid::DataGrid(const DataGrid &r) { memcpy((void *)this, (const void *)&r, sizeof(DataGrid)); }
DataGrid::~DataGrid() {}
void DataGrid::set_gdims(int gdims[3]) {
  for (int i = 0; i < 3; i++) {
    Gdims[i] = gdims[i];
    Ldims[i] = gdims[i];
  }
}

trans_type3D::trans_type3D(int types_IDs[3]) {
  p3d::ensure_setup();
  name = nullptr;
  is_set = true;
  for (int i = 0; i < 3; i++) {
    if (types_IDs[i] < 0 || types_IDs[i] >= 44) {
      cout << "Error in init trans_plan: type is undefined " << types_IDs[i] << endl;
      is_set = false;
    }
    types[i] = types_IDs[i];
  }
  prec = is_set ? p3d::g_types[types[0]].prec : 0;
}
trans_type3D::trans_type3D(const trans_type3D &r) {
  name = nullptr;
  is_set = r.is_set;
  prec = r.prec;
  for (int i = 0; i < 3; i++) types[i] = r.types[i];
}
trans_type3D::~trans_type3D() {}

void timer::init() {
  p3dfft_gb300_reset_timers();
  p3dfft_gb300_enable_timers(1);
  reorder_deriv = reorder_trans = reorder_out = reorder_in = trans_exec = trans_deriv = 0;
  packsend = packsend_trans = packsend_deriv = unpackrecv = alltoall = 0;
}
void timer::print(MPI_Comm) {
  trans_exec = p3dfft_gb300_timer(0);
  reorder_trans = p3dfft_gb300_timer(1);
  reorder_out = p3dfft_gb300_timer(2);
  trans_deriv = p3dfft_gb300_timer(3);
  printf("P3DFFT++ (GB300) timers (device seconds): trans_exec=%lg reorder_trans=%lg reorder_out=%lg "
         "trans_deriv=%lg h2d=%lg d2h=%lg\n",
         trans_exec, reorder_trans, reorder_out, trans_deriv, p3dfft_gb300_timer(4), p3dfft_gb300_timer(5));
}

}  // namespace p3dfft
