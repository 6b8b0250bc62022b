/*
 * p3d_oracle.h -- CPU oracle for the P3DFFT++ 3D transform pipeline on a 1x1x1 processor grid.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference algorithm, used as
 * the checker by tests/, by __graft_entry__.smoke() and by bench.py's cpu_baseline / reference
 * arm.  The product library (libp3dfft_gb300.so) never links, loads or calls it.
 *
 * Parity pin: the reference's 1D arithmetic lives in FFTW 3 (not vendored, version unpinned;
 * call sites build/init.C:1146-1188, 1191-1607).  The oracle restates FFTW's published
 * transform definitions and is pinned by (a) the analytic known-answer checks of the
 * reference's own sample programs (sample/C++/test3D_r2c.C, test_deriv.C, test1D_cos.C,
 * test1D_sin.C, test3D_c2c.C), (b) an O(n^2) long-double direct DFT for small n, and
 * (c) scipy.fft (pocketfft) in the CPU test-suite.  See tests/test_oracle_*.py.
 *
 * All arithmetic is double precision; twiddle / trig tables are generated in long double.
 */
#ifndef P3D_ORACLE_H
#define P3D_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Transform type IDs 0..43, in the registration order of p3dfft::setup()
 * (build/init.C:121-731). */
enum {
  ORC_NTYPES = 44
};

/* Per-type description (build/init.C:121-731, 2089-2182). kind values below. */
enum {
  ORC_K_EMPTY = 0,
  ORC_K_R2C = 1,
  ORC_K_C2R = 2,
  ORC_K_C2C_FWD = 3,
  ORC_K_C2C_BWD = 4,
  ORC_K_R2R = 5 /* r2r kind in .r2r, applied to re/im separately when dt1 == dt2 == 2 */
};
/* FFTW r2r kinds (public FFTW 3 manual) */
enum { ORC_REDFT00 = 0, ORC_REDFT10, ORC_REDFT01, ORC_REDFT11,
       ORC_RODFT00, ORC_RODFT10, ORC_RODFT01, ORC_RODFT11 };

typedef struct {
  int dt1, dt2;  /* 1 = real, 2 = complex */
  int prec;      /* 4 or 8 */
  int kind;      /* ORC_K_* */
  int r2r;       /* ORC_REDFT00.. when kind == ORC_K_R2R */
} orc_type_info;

int orc_type_info_get(int type_id, orc_type_info *out);

/* ---- 1D arithmetic on contiguous double lines ---- */
/* complex DFT, out[k] = sum_j in[j] exp(sign*2*pi*i*j*k/n); interleaved re/im */
void orc_dft_c2c(int n, int sign, const double *in, double *out);
/* real -> half complex (n/2+1 outputs), forward sign -1, unnormalised */
void orc_dft_r2c(int n, const double *in, double *out);
/* half complex (n/2+1 inputs) -> real n, sign +1, imag parts of DC / Nyquist ignored */
void orc_dft_c2r(int n, const double *in, double *out);
/* FFTW r2r kind on a real line of length n (unnormalised FFTW definitions) */
void orc_r2r(int kind, int n, const double *in, double *out);
/* O(n^2) long-double direct DFT for self-checks */
void orc_dft_direct(int n, int sign, const double *in, double *out);

/* Reusable plan for many lines of one transform: kind ORC_K_*, r2r kind for ORC_K_R2R, logical
 * length n.  orc_line_exec runs one contiguous line (complex = interleaved pairs; in and out must
 * not overlap) with `work` holding orc_line_work_doubles() doubles.  NULL for an invalid kind or
 * length. */
typedef struct orc_line orc_line;
orc_line *orc_line_new(int kind, int r2r, int n);
size_t orc_line_work_doubles(const orc_line *L);
void orc_line_exec(const orc_line *L, const double *in, double *out, double *work);
void orc_line_free(orc_line *L);

/* ---- Planner (1x1x1 processor grid) ---- */
typedef struct {
  int gdims[3];  /* global == local dims on one rank */
  int mo[3];     /* MemOrder: storage rank of logical dim d, 0 = stride-1 */
  int dcs;       /* dim_conj_sym, -1 if none */
} orc_grid;

typedef struct {
  int type;      /* 1D type id, possibly an EMPTY type */
  int dim;       /* trans_dim */
  orc_grid g1, g2;
} orc_stage;

#define ORC_MAX_STAGES 4
typedef struct {
  int nstages;
  orc_stage st[ORC_MAX_STAGES];
  int L[3];
  int dt1, dt2, prec;
  int ok;
} orc_plan3d;

/* 1 (default): stages of C2C lines, and R2C / C2R lines of even length, run on the batched
 * line engine (blocks of 16 lines, vectorised butterflies); 0: line by line.  Same results to
 * rounding. */
void orc_set_batched(int on);

/* Builds the stage list of transform3D<T1,T2>::transform3D (build/templ.C:91-420). Returns 0 on
 * success, nonzero on an error the reference would print. */
int orc_plan3d_make(const int types[3], const orc_grid *g1, const orc_grid *g2, orc_plan3d *p);
/* Executes the plan (build/exec.C:101-223). Element type follows dt1/dt2 of the plan, always in
 * double precision (complex = interleaved pairs).  idir = -1 for plain exec, else the logical
 * dimension of the spectral derivative. nthreads <= 0 -> all available (OpenMP). */
int orc_exec3d(const orc_plan3d *p, const double *in, double *out, int idir, int nthreads);
/* One 1D stage (transplan::exec, build/exec.C:522-622) on explicit grids. */
int orc_exec_stage(const orc_stage *s, const double *in, double *out, int deriv, int nthreads);
/* Same, restricted to lines [line0, line1) of the stage (line = index over the two batch dims,
 * first batch dim fastest; on the batched engine the batch dim with the smaller input stride
 * fastest); line1 < 0 means all lines.  Used to time bounded samples. */
int orc_exec_stage_lines(const orc_stage *s, const double *in, double *out, int deriv, int nthreads,
                         long long line0, long long line1);
/* Standalone spectral derivative (build/deriv.C:85-184) on a complex field, along logical dim
 * idir.  orc_compute_deriv_axis with ref_axis = 1 differentiates along the storage axis the
 * reference uses (rank imo[idir], deriv.C:89-93), which differs for the 3-cycle memory orders. */
int orc_compute_deriv(const orc_grid *g, const double *in, double *out, int idir);
int orc_compute_deriv_axis(const orc_grid *g, const double *in, double *out, int idir, int ref_axis);

/* helpers exposed for tests */
void orc_swap0(int newmo[3], const int mo[3], int L);
int orc_find_order(const int types[3], const orc_grid *g1, const orc_grid *g2, int L[3]);
long long orc_grid_elems(const orc_grid *g);

#ifdef __cplusplus
}
#endif
#endif
