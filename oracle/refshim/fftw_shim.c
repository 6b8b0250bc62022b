/*
 * fftw_shim.c -- the FFTW 3 entry points of refshim/fftw3.h on the oracle's 1D arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/libp3dfft_ref.so together with the
 * reference's own build/{init,templ,exec,deriv,wrap}.C, compiled unchanged, so that the reference
 * driver (planner, memory-order reorders, derivative, C wrappers) can be run here as a parity
 * anchor.  The product library never links it.
 *
 * Semantics follow the FFTW 3 manual for rank-1 "many" plans:
 *   element j of transform k sits at in[k*idist + j*istride] (out likewise, with ostride/odist),
 *   in units of the array's element type (fftw_complex for complex arrays);
 *   c2c: out_k = sum_j in_j exp(sign 2 pi i j k / n), unnormalised;
 *   r2c: n reals -> n/2+1 complex, sign -1;  c2r: n/2+1 complex -> n reals, sign +1, the
 *   imaginary parts of DC and (even n) Nyquist ignored;  r2r: the REDFT/RODFT kinds as defined in
 *   "What FFTW Really Computes".
 * The arithmetic is the oracle's (double precision, long-double twiddles); single-precision plans
 * convert to double and round the result.  Plans never touch the arrays they are made with
 * (FFTW_ESTIMATE behaviour).  Arrays that overlap (in-place execution) are gathered in full before
 * any output is written, so every layout FFTW accepts gives FFTW's result.  Lines run in parallel
 * with OpenMP when the arrays do not overlap.
 */
#include "fftw3.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../p3d_oracle.h"

enum { W_C2C, W_R2C, W_C2R, W_R2R };

struct orc_fftw_plan_s {
  int what, n, howmany, istride, idist, ostride, odist, prec;
  int nin, nout, cin, cout; /* points per line in / out; 1 = complex elements */
  orc_line *line;
};

void *fftw_malloc(size_t n)
{
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 1)) return NULL;
  return p;
}
void fftw_free(void *p) { free(p); }
void fftw_destroy_plan(fftw_plan p)
{
  if (!p) return;
  orc_line_free(p->line);
  free(p);
}
void fftwf_destroy_plan(fftwf_plan p) { fftw_destroy_plan(p); }
void fftw_cleanup(void) {}
void fftwf_cleanup(void) {}

static int orc_kind_of(fftw_r2r_kind k)
{
  switch (k) {
    case FFTW_REDFT00: return ORC_REDFT00;
    case FFTW_REDFT10: return ORC_REDFT10;
    case FFTW_REDFT01: return ORC_REDFT01;
    case FFTW_REDFT11: return ORC_REDFT11;
    case FFTW_RODFT00: return ORC_RODFT00;
    case FFTW_RODFT10: return ORC_RODFT10;
    case FFTW_RODFT01: return ORC_RODFT01;
    case FFTW_RODFT11: return ORC_RODFT11;
    default: return -1;
  }
}

static struct orc_fftw_plan_s *make(int what, int prec, int rank, const int *n, int howmany, int istride,
                                    int idist, int ostride, int odist, int sign, int r2r)
{
  struct orc_fftw_plan_s *p;
  int kind;
  if (rank != 1 || !n || n[0] < 1 || howmany < 0) return NULL;
  switch (what) {
    case W_C2C: kind = (sign < 0) ? ORC_K_C2C_FWD : ORC_K_C2C_BWD; break;
    case W_R2C: kind = ORC_K_R2C; break;
    case W_C2R: kind = ORC_K_C2R; break;
    default:
      kind = ORC_K_R2R;
      if (r2r < 0) return NULL;
  }
  p = (struct orc_fftw_plan_s *)calloc(1, sizeof(*p));
  p->line = orc_line_new(kind, r2r < 0 ? 0 : r2r, n[0]);
  if (!p->line) {
    free(p);
    return NULL;
  }
  p->what = what;
  p->prec = prec;
  p->n = n[0];
  p->howmany = howmany;
  p->istride = istride;
  p->idist = idist;
  p->ostride = ostride;
  p->odist = odist;
  p->nin = (what == W_C2R) ? n[0] / 2 + 1 : n[0];
  p->nout = (what == W_R2C) ? n[0] / 2 + 1 : n[0];
  p->cin = (what == W_C2C || what == W_C2R);
  p->cout = (what == W_C2C || what == W_R2C);
  return p;
}

/* Byte range [lo, hi) touched by one array of the plan. */
static void span(const void *base, int howmany, int nper, int stride, int dist, size_t esz, uintptr_t *lo,
                 uintptr_t *hi)
{
  long long first = 0, last = 0, a = (long long)(howmany - 1) * dist, b = (long long)(nper - 1) * stride;
  if (a < 0) first += a; else last += a;
  if (b < 0) first += b; else last += b;
  *lo = (uintptr_t)base + (uintptr_t)(first * (long long)esz);
  *hi = (uintptr_t)base + (uintptr_t)((last + 1) * (long long)esz);
}

static void gather(const struct orc_fftw_plan_s *p, const void *in, int k, double *line)
{
  int j, w = p->cin ? 2 : 1;
  for (j = 0; j < p->nin; j++) {
    long long e = (long long)k * p->idist + (long long)j * p->istride;
    int c;
    for (c = 0; c < w; c++)
      line[w * j + c] = (p->prec == 8) ? ((const double *)in)[w * e + c] : (double)((const float *)in)[w * e + c];
  }
}

static void scatter(const struct orc_fftw_plan_s *p, const double *line, int k, void *out)
{
  int j, w = p->cout ? 2 : 1;
  for (j = 0; j < p->nout; j++) {
    long long e = (long long)k * p->odist + (long long)j * p->ostride;
    int c;
    for (c = 0; c < w; c++) {
      if (p->prec == 8) ((double *)out)[w * e + c] = line[w * j + c];
      else ((float *)out)[w * e + c] = (float)line[w * j + c];
    }
  }
}

static void run(const struct orc_fftw_plan_s *p, const void *in, void *out)
{
  size_t esz, inw, outw, wk;
  int overlap, k;
  uintptr_t a0, a1, b0, b1;
  if (!p || p->howmany == 0) return;
  esz = (size_t)p->prec;
  inw = 2 * (size_t)p->nin + 2;
  outw = 2 * (size_t)p->nout + 2;
  wk = orc_line_work_doubles(p->line);
  span(in, p->howmany, p->nin, p->istride, p->idist, esz * (p->cin ? 2 : 1), &a0, &a1);
  span(out, p->howmany, p->nout, p->ostride, p->odist, esz * (p->cout ? 2 : 1), &b0, &b1);
  overlap = (a0 < b1 && b0 < a1);
  if (overlap) {
    /* in-place: read every line before writing any */
    double *all = (double *)malloc(sizeof(double) * inw * (size_t)p->howmany);
    double *o = (double *)malloc(sizeof(double) * (outw + wk));
    if (!all || !o) {
      fprintf(stderr, "fftw shim: out of memory\n");
      abort();
    }
    for (k = 0; k < p->howmany; k++) gather(p, in, k, all + inw * (size_t)k);
    for (k = 0; k < p->howmany; k++) {
      orc_line_exec(p->line, all + inw * (size_t)k, o, o + outw);
      scatter(p, o, k, out);
    }
    free(all);
    free(o);
    return;
  }
#pragma omp parallel if (p->howmany >= 64)
  {
    double *buf = (double *)malloc(sizeof(double) * (inw + outw + wk));
#pragma omp for schedule(static)
    for (k = 0; k < p->howmany; k++) {
      gather(p, in, k, buf);
      orc_line_exec(p->line, buf, buf + inw, buf + inw + outw);
      scatter(p, buf + inw, k, out);
    }
    free(buf);
  }
}

/* ---- double precision ---- */
fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                             int istride, int idist, fftw_complex *out, const int *onembed, int ostride,
                             int odist, int sign, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_C2C, 8, rank, n, howmany, istride, idist, ostride, odist, sign, -1);
}
fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in, const int *inembed,
                                 int istride, int idist, fftw_complex *out, const int *onembed,
                                 int ostride, int odist, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_R2C, 8, rank, n, howmany, istride, idist, ostride, odist, -1, -1);
}
fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                                 int istride, int idist, double *out, const int *onembed, int ostride,
                                 int odist, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_C2R, 8, rank, n, howmany, istride, idist, ostride, odist, +1, -1);
}
fftw_plan fftw_plan_many_r2r(int rank, const int *n, int howmany, double *in, const int *inembed,
                             int istride, int idist, double *out, const int *onembed, int ostride,
                             int odist, const fftw_r2r_kind *kind, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_R2R, 8, rank, n, howmany, istride, idist, ostride, odist, 0, kind ? orc_kind_of(kind[0]) : -1);
}
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) { run(p, in, out); }
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out) { run(p, in, out); }
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out) { run(p, in, out); }
void fftw_execute_r2r(const fftw_plan p, double *in, double *out) { run(p, in, out); }

/* ---- single precision ---- */
fftwf_plan fftwf_plan_many_dft(int rank, const int *n, int howmany, fftwf_complex *in, const int *inembed,
                               int istride, int idist, fftwf_complex *out, const int *onembed,
                               int ostride, int odist, int sign, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_C2C, 4, rank, n, howmany, istride, idist, ostride, odist, sign, -1);
}
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int *n, int howmany, float *in, const int *inembed,
                                   int istride, int idist, fftwf_complex *out, const int *onembed,
                                   int ostride, int odist, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_R2C, 4, rank, n, howmany, istride, idist, ostride, odist, -1, -1);
}
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int *n, int howmany, fftwf_complex *in,
                                   const int *inembed, int istride, int idist, float *out,
                                   const int *onembed, int ostride, int odist, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_C2R, 4, rank, n, howmany, istride, idist, ostride, odist, +1, -1);
}
fftwf_plan fftwf_plan_many_r2r(int rank, const int *n, int howmany, float *in, const int *inembed,
                               int istride, int idist, float *out, const int *onembed, int ostride,
                               int odist, const fftwf_r2r_kind *kind, unsigned flags)
{
  (void)in; (void)out; (void)inembed; (void)onembed; (void)flags;
  return make(W_R2R, 4, rank, n, howmany, istride, idist, ostride, odist, 0, kind ? orc_kind_of(kind[0]) : -1);
}
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) { run(p, in, out); }
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out) { run(p, in, out); }
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out) { run(p, in, out); }
void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out) { run(p, in, out); }
