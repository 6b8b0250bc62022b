/*
 * p3d_oracle.c -- CPU oracle for the P3DFFT++ 3D transform pipeline (1x1x1 processor grid).
 *
 * TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke() and bench.py's
 * CPU baseline.  The product library never links or calls this file.
 *
 * Restates, in plain C and in double precision:
 *   - the 1D type registry of p3dfft::setup()            (build/init.C:121-731)
 *   - FFTW 3's published transform definitions that the reference delegates to
 *     (execute adaptors build/init.C:1146-1188, planners build/init.C:1191-1607)
 *   - the 3D planner: find_order / swap0 / excl / stage loop / final_seq
 *                                                        (build/templ.C:91-435, 627-882)
 *   - the stage executor and fused derivative             (build/exec.C:101-287, 522-702)
 *   - the standalone spectral derivative                  (build/deriv.C:85-184)
 * Memory layouts, stage order and derivative wavenumbers follow the reference exactly; the
 * buffer ping-pong of exec.C:127-166 is replaced by plain temporaries (it does not change
 * results).  Deviations from the reference's literal behaviour are limited to its defects
 * and are marked QUIRK below, each with the reference line it concerns.
 */
#include "p3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------ */
/* Type registry: build/init.C:121-731.  IDs: 0-3 EMPTY (S, D, S complex, D complex),
 * 4 R2C_S, 5 R2C_D, 6 C2R_S, 7 C2R_D, 8 CFFT_FORWARD_S, 9 CFFT_FORWARD_D, 10 CFFT_BACKWARD_S,
 * 11 CFFT_BACKWARD_D, then for each of DCT1, DST1, DCT2, DST2, DCT3, DST3, DCT4, DST4 the four
 * variants REAL_S, REAL_D, COMPLEX_S, COMPLEX_D (IDs 12..43).
 * QUIRK (reproduced): the DCT4 IDs are registered with the DCT1 planners
 * (build/init.C:640, 652, 664, 676), so they compute REDFT00. */
int orc_type_info_get(int id, orc_type_info *o)
{
  static const int r2r_of_family[8] = {ORC_REDFT00, ORC_RODFT00, ORC_REDFT10, ORC_RODFT10,
                                       ORC_REDFT01, ORC_RODFT01, ORC_REDFT00 /* DCT4 quirk */,
                                       ORC_RODFT11};
  if (id < 0 || id >= ORC_NTYPES) return -1;
  memset(o, 0, sizeof(*o));
  if (id < 4) {
    o->kind = ORC_K_EMPTY;
    o->prec = (id & 1) ? 8 : 4;
    o->dt1 = o->dt2 = (id >= 2) ? 2 : 1;
    return 0;
  }
  if (id < 12) {
    int j = id - 4;
    o->prec = (j & 1) ? 8 : 4;
    switch (j >> 1) {
      case 0: o->kind = ORC_K_R2C; o->dt1 = 1; o->dt2 = 2; break;
      case 1: o->kind = ORC_K_C2R; o->dt1 = 2; o->dt2 = 1; break;
      case 2: o->kind = ORC_K_C2C_FWD; o->dt1 = o->dt2 = 2; break;
      default: o->kind = ORC_K_C2C_BWD; o->dt1 = o->dt2 = 2; break;
    }
    return 0;
  }
  {
    int j = id - 12, fam = j / 4, var = j % 4;
    o->kind = ORC_K_R2R;
    o->r2r = r2r_of_family[fam];
    o->prec = (var & 1) ? 8 : 4;
    o->dt1 = o->dt2 = (var >= 2) ? 2 : 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Complex DFT of any length: recursive mixed-radix decimation in time, twiddles from a long
 * double table.  Prime factors > 7 use a direct O(p^2) butterfly. */
typedef struct {
  int n;
  int nf;
  int fac[40];
  double *w; /* w[2k], w[2k+1] = cos(2 pi k/n), -sin(2 pi k/n) */
  int maxp;
} fftplan;

static void fftplan_init(fftplan *P, int n)
{
  static const long double TWO_PI = 6.283185307179586476925286766559005768L;
  int m = n, k;
  P->n = n;
  P->nf = 0;
  P->maxp = 1;
  while (m > 1) {
    int p;
    if (m % 4 == 0) p = 4;
    else if (m % 2 == 0) p = 2;
    else {
      for (p = 3; p * p <= m; p += 2)
        if (m % p == 0) break;
      if (p * p > m) p = m;
    }
    P->fac[P->nf++] = p;
    if (p > P->maxp) P->maxp = p;
    m /= p;
  }
  P->w = (double *)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
  for (k = 0; k < n; k++) {
    long double a = TWO_PI * (long double)k / (long double)n;
    P->w[2 * k] = (double)cosl(a);
    P->w[2 * k + 1] = (double)-sinl(a);
  }
}
static void fftplan_free(fftplan *P) { free(P->w); }

static void fft_rec(const fftplan *P, int n, int sw, const double *in, int is, double *out,
                    int fi, int sign, double *t)
{
  int p, m, r, k, q, N = P->n;
  if (n == 1) {
    out[0] = in[0];
    out[1] = in[1];
    return;
  }
  p = P->fac[fi];
  m = n / p;
  for (r = 0; r < p; r++) fft_rec(P, m, sw * p, in + 2 * (size_t)r * is, is * p, out + 2 * (size_t)r * m, fi + 1, sign, t);
  for (k = 0; k < m; k++) {
    for (r = 0; r < p; r++) {
      int wi = r * k * sw; /* < N */
      double wr = P->w[2 * wi], wim = sign < 0 ? P->w[2 * wi + 1] : -P->w[2 * wi + 1];
      double yr = out[2 * (k + r * m)], yi = out[2 * (k + r * m) + 1];
      t[2 * r] = yr * wr - yi * wim;
      t[2 * r + 1] = yr * wim + yi * wr;
    }
    for (q = 0; q < p; q++) {
      double sr = 0, si = 0;
      for (r = 0; r < p; r++) {
        int wi = (int)(((long long)r * q % p) * (N / p));
        double wr = P->w[2 * wi], wim = sign < 0 ? P->w[2 * wi + 1] : -P->w[2 * wi + 1];
        sr += t[2 * r] * wr - t[2 * r + 1] * wim;
        si += t[2 * r] * wim + t[2 * r + 1] * wr;
      }
      out[2 * (k + q * m)] = sr;
      out[2 * (k + q * m) + 1] = si;
    }
  }
}

static void fft_exec(const fftplan *P, int sign, const double *in, double *out, double *t)
{
  fft_rec(P, P->n, 1, in, 1, out, 0, sign, t);
}

void orc_dft_c2c(int n, int sign, const double *in, double *out)
{
  fftplan P;
  double *t, *o;
  if (n <= 0) return;
  fftplan_init(&P, n);
  t = (double *)malloc(sizeof(double) * 2 * P.maxp);
  o = (double *)malloc(sizeof(double) * 2 * n);
  fft_exec(&P, sign, in, o, t);
  memcpy(out, o, sizeof(double) * 2 * n);
  free(o);
  free(t);
  fftplan_free(&P);
}

void orc_dft_direct(int n, int sign, const double *in, double *out)
{
  static const long double TWO_PI = 6.283185307179586476925286766559005768L;
  int j, k;
  for (k = 0; k < n; k++) {
    long double sr = 0, si = 0;
    for (j = 0; j < n; j++) {
      long long jk = ((long long)j * k) % n;
      long double a = TWO_PI * (long double)jk / (long double)n;
      long double c = cosl(a), s = sign * sinl(a);
      sr += in[2 * j] * c - in[2 * j + 1] * s;
      si += in[2 * j] * s + in[2 * j + 1] * c;
    }
    out[2 * k] = (double)sr;
    out[2 * k + 1] = (double)si;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Line transforms with reusable per-thread workspaces. */
typedef struct {
  int kind, r2r, n;   /* logical length n (real length for R2C/C2R) */
  fftplan P;          /* complex plan of length n (FFT kinds) */
  double *cs;         /* r2r: trig table, cs[2t] = cos(2 pi t/M), cs[2t+1] = sin(2 pi t/M) */
  int M;
} lineplan;

static void lineplan_init(lineplan *L, int kind, int r2r, int n)
{
  static const long double TWO_PI = 6.283185307179586476925286766559005768L;
  int t;
  memset(L, 0, sizeof(*L));
  L->kind = kind;
  L->r2r = r2r;
  L->n = n;
  if (kind == ORC_K_EMPTY) return;
  if (kind != ORC_K_R2R) {
    fftplan_init(&L->P, n);
    return;
  }
  switch (r2r) {
    case ORC_REDFT00: L->M = 2 * (n - 1); break;
    case ORC_RODFT00: L->M = 2 * (n + 1); break;
    case ORC_REDFT11:
    case ORC_RODFT11: L->M = 8 * n; break;
    default: L->M = 4 * n; break;
  }
  if (L->M < 1) L->M = 1;
  L->cs = (double *)malloc(sizeof(double) * 2 * L->M);
  for (t = 0; t < L->M; t++) {
    long double a = TWO_PI * (long double)t / (long double)L->M;
    L->cs[2 * t] = (double)cosl(a);
    L->cs[2 * t + 1] = (double)sinl(a);
  }
}
static void lineplan_free(lineplan *L)
{
  if (L->kind != ORC_K_EMPTY && L->kind != ORC_K_R2R) fftplan_free(&L->P);
  free(L->cs);
}

/* FFTW r2r definitions (FFTW 3 manual, "What FFTW Really Computes"), real line in -> out.
 * in/out strides in doubles (2 for the complex variants, exec_r2r_complex_* at
 * build/init.C:1179-1188). */
static void r2r_line(const lineplan *L, const double *in, int is, double *out, int os)
{
  int n = L->n, M = L->M, j, k;
  const double *cs = L->cs;
#define C_(t) cs[2 * (int)(((long long)(t)) % M)]
#define S_(t) cs[2 * (int)(((long long)(t)) % M) + 1]
  for (k = 0; k < n; k++) {
    double s = 0;
    switch (L->r2r) {
      case ORC_REDFT00: /* Y_k = X_0 + (-1)^k X_{n-1} + 2 sum_{j=1}^{n-2} X_j cos(pi j k/(n-1)) */
        if (n == 1) { s = in[0]; break; }
        s = in[0] + ((k & 1) ? -in[(size_t)(n - 1) * is] : in[(size_t)(n - 1) * is]);
        for (j = 1; j < n - 1; j++) s += 2.0 * in[(size_t)j * is] * C_((long long)j * k);
        break;
      case ORC_REDFT10: /* 2 sum X_j cos(pi (j+1/2) k / n) */
        for (j = 0; j < n; j++) s += in[(size_t)j * is] * C_((long long)(2 * j + 1) * k);
        s *= 2.0;
        break;
      case ORC_REDFT01: /* X_0 + 2 sum_{j>=1} X_j cos(pi j (k+1/2)/n) */
        for (j = 1; j < n; j++) s += in[(size_t)j * is] * C_((long long)j * (2 * k + 1));
        s = in[0] + 2.0 * s;
        break;
      case ORC_REDFT11: /* 2 sum X_j cos(pi (j+1/2)(k+1/2)/n) */
        for (j = 0; j < n; j++) s += in[(size_t)j * is] * C_((long long)(2 * j + 1) * (2 * k + 1));
        s *= 2.0;
        break;
      case ORC_RODFT00: /* 2 sum X_j sin(pi (j+1)(k+1)/(n+1)) */
        for (j = 0; j < n; j++) s += in[(size_t)j * is] * S_((long long)(j + 1) * (k + 1));
        s *= 2.0;
        break;
      case ORC_RODFT10: /* 2 sum X_j sin(pi (j+1/2)(k+1)/n) */
        for (j = 0; j < n; j++) s += in[(size_t)j * is] * S_((long long)(2 * j + 1) * (k + 1));
        s *= 2.0;
        break;
      case ORC_RODFT01: /* (-1)^k X_{n-1} + 2 sum_{j=0}^{n-2} X_j sin(pi (j+1)(k+1/2)/n) */
        for (j = 0; j < n - 1; j++) s += in[(size_t)j * is] * S_((long long)(j + 1) * (2 * k + 1));
        s = 2.0 * s + ((k & 1) ? -in[(size_t)(n - 1) * is] : in[(size_t)(n - 1) * is]);
        break;
      case ORC_RODFT11: /* 2 sum X_j sin(pi (j+1/2)(k+1/2)/n) */
        for (j = 0; j < n; j++) s += in[(size_t)j * is] * S_((long long)(2 * j + 1) * (2 * k + 1));
        s *= 2.0;
        break;
    }
    out[(size_t)k * os] = s;
  }
#undef C_
#undef S_
}

void orc_r2r(int kind, int n, const double *in, double *out)
{
  lineplan L;
  double *o = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  lineplan_init(&L, ORC_K_R2R, kind, n);
  r2r_line(&L, in, 1, o, 1);
  memcpy(out, o, sizeof(double) * n);
  free(o);
  lineplan_free(&L);
}

/* work: >= 4*n + 2*maxp doubles */
static void r2c_line(const lineplan *L, const double *in, double *out, double *work)
{
  int n = L->n, j;
  double *a = work, *b = work + 2 * n, *t = work + 4 * n;
  for (j = 0; j < n; j++) {
    a[2 * j] = in[j];
    a[2 * j + 1] = 0.0;
  }
  fft_exec(&L->P, -1, a, b, t);
  memcpy(out, b, sizeof(double) * 2 * (n / 2 + 1));
}

/* c2r: Hermitian extension of the n/2+1 inputs; the imaginary parts of DC and (n even)
 * Nyquist are ignored (they do not contribute to a real output). */
static void c2r_line(const lineplan *L, const double *in, double *out, double *work)
{
  int n = L->n, h = n / 2 + 1, k;
  double *a = work, *b = work + 2 * n, *t = work + 4 * n;
  for (k = 0; k < h; k++) {
    a[2 * k] = in[2 * k];
    a[2 * k + 1] = in[2 * k + 1];
  }
  a[1] = 0.0;
  if ((n & 1) == 0) a[2 * (n / 2) + 1] = 0.0;
  for (k = h; k < n; k++) {
    a[2 * k] = a[2 * (n - k)];
    a[2 * k + 1] = -a[2 * (n - k) + 1];
  }
  fft_exec(&L->P, +1, a, b, t);
  for (k = 0; k < n; k++) out[k] = b[2 * k];
}

void orc_dft_r2c(int n, const double *in, double *out)
{
  lineplan L;
  double *w = (double *)malloc(sizeof(double) * (4 * (size_t)n + 64 + 2 * (size_t)n));
  lineplan_init(&L, ORC_K_R2C, 0, n);
  r2c_line(&L, in, out, w);
  free(w);
  lineplan_free(&L);
}

void orc_dft_c2r(int n, const double *in, double *out)
{
  lineplan L;
  double *w = (double *)malloc(sizeof(double) * (4 * (size_t)n + 64 + 2 * (size_t)n));
  lineplan_init(&L, ORC_K_C2R, 0, n);
  c2r_line(&L, in, out, w);
  free(w);
  lineplan_free(&L);
}

/* Reusable line plans for callers that run many lines of one transform (the FFTW-API shim of
 * oracle/refshim/fftw_shim.c, through which the reference's own driver runs on this arithmetic). */
struct orc_line {
  lineplan L;
  int maxp;
};

orc_line *orc_line_new(int kind, int r2r, int n)
{
  orc_line *P;
  if (n < 1 || kind < ORC_K_EMPTY || kind > ORC_K_R2R) return NULL;
  if (kind == ORC_K_R2R && ((r2r == ORC_REDFT00 && n < 2) || r2r < ORC_REDFT00 || r2r > ORC_RODFT11)) return NULL;
  P = (orc_line *)calloc(1, sizeof(*P));
  lineplan_init(&P->L, kind, r2r, n);
  P->maxp = (kind != ORC_K_EMPTY && kind != ORC_K_R2R) ? P->L.P.maxp : 1;
  return P;
}

size_t orc_line_work_doubles(const orc_line *P) { return 6 * (size_t)P->L.n + 2 * (size_t)P->maxp + 72; }

void orc_line_exec(const orc_line *P, const double *in, double *out, double *work)
{
  const lineplan *L = &P->L;
  switch (L->kind) {
    case ORC_K_EMPTY: memcpy(out, in, sizeof(double) * L->n); break;
    case ORC_K_R2C: r2c_line(L, in, out, work); break;
    case ORC_K_C2R: c2r_line(L, in, out, work); break;
    case ORC_K_C2C_FWD: fft_exec(&L->P, -1, in, out, work); break;
    case ORC_K_C2C_BWD: fft_exec(&L->P, +1, in, out, work); break;
    case ORC_K_R2R: r2r_line(L, in, 1, out, 1); break;
  }
}

void orc_line_free(orc_line *P)
{
  if (!P) return;
  lineplan_free(&P->L);
  free(P);
}

/* compute_deriv_loc, build/exec.C:228-287, on one complex line of length M (M = output length
 * of the stage's transform).  r2c lines use g = 2(M-1) (exec.C:240-243). */
static void deriv_line(double *x, int M, int r2c)
{
  int g = r2c ? (M - 1) * 2 : M, mid = g / 2, i;
  for (i = 0; i < M; i++) {
    double k, re = x[2 * i], im = x[2 * i + 1];
    if (i < mid) k = (double)i;
    else if (i == mid) { x[2 * i] = 0.0; x[2 * i + 1] = 0.0; continue; }
    else k = (double)(i - g);
    x[2 * i] = -k * im;
    x[2 * i + 1] = k * re;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Batched line engine (the same definitions as fft_rec / r2c_line / c2r_line, computed B lines at
 * a time): the lines are gathered into split re / im arrays with the line index fastest, so that
 * every butterfly is a loop over B lines that the compiler vectorises, and a stage's lines are
 * taken in blocks of B neighbours in memory.  Stockham passes of radix 4, 2 and 3, any other
 * factor as a direct DFT of its length; twiddles from long double tables.  Used by the stage
 * executor for C2C lines of any length and R2C / C2R lines of even length (half-length complex
 * FFT with the standard even / odd split); results agree with the per-line path to rounding. */
#define ORC_NB 16
static int g_batched = 1;
void orc_set_batched(int on) { g_batched = on ? 1 : 0; }

typedef struct {
  int h;            /* complex FFT length */
  int ts;           /* table stride: the table holds N = h * ts points */
  int nf, fac[40];
  double *wr, *wi;  /* wr[t] = cos(2 pi t / N), wi[t] = -sin(2 pi t / N), t < N */
} bplan;

static void bplan_init(bplan *P, int h, int ts)
{
  static const long double TWO_PI = 6.283185307179586476925286766559005768L;
  int m = h, t, N = h * ts;
  P->h = h;
  P->ts = ts;
  P->nf = 0;
  while (m > 1) {
    int p;
    if (m % 4 == 0) p = 4;
    else if (m % 2 == 0) p = 2;
    else if (m % 3 == 0) p = 3;
    else {
      for (p = 5; p * p <= m; p += 2)
        if (m % p == 0) break;
      if (p * p > m) p = m;
    }
    P->fac[P->nf++] = p;
    m /= p;
  }
  P->wr = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
  P->wi = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
  for (t = 0; t < N; t++) {
    long double a = TWO_PI * (long double)t / (long double)N;
    P->wr[t] = (double)cosl(a);
    P->wi[t] = (double)-sinl(a);
  }
}
static void bplan_free(bplan *P)
{
  free(P->wr);
  free(P->wi);
}

/* One Stockham pass of radix p: y[q + s(p pp + t)] = W^(t pp s) sum_r x[q + s(pp + r m)] w_p^(rt),
 * W = exp(sign 2 pi i / h), for pp < m, q < s; element i is the B values at [i B, i B + B). */
static void bpass(const bplan *P, int p, int m, int s, int sign, const double *restrict xr,
                  const double *restrict xi, double *restrict yr, double *restrict yi)
{
  const int ts = P->ts, N = P->h * ts;
  const double sg = sign < 0 ? 1.0 : -1.0; /* the table holds the forward (sign -1) angles */
  int pp, q, l, r, t;
  for (pp = 0; pp < m; pp++) {
    for (q = 0; q < s; q++) {
      const size_t i0 = (size_t)(q + s * pp);
      const size_t o0 = (size_t)(q + s * p * pp);
      if (p == 4) {
        const double *a0r = xr + i0 * ORC_NB, *a0i = xi + i0 * ORC_NB;
        const double *a1r = xr + (i0 + (size_t)s * m) * ORC_NB, *a1i = xi + (i0 + (size_t)s * m) * ORC_NB;
        const double *a2r = xr + (i0 + (size_t)2 * s * m) * ORC_NB, *a2i = xi + (i0 + (size_t)2 * s * m) * ORC_NB;
        const double *a3r = xr + (i0 + (size_t)3 * s * m) * ORC_NB, *a3i = xi + (i0 + (size_t)3 * s * m) * ORC_NB;
        double *y0r = yr + o0 * ORC_NB, *y0i = yi + o0 * ORC_NB;
        double *y1r = yr + (o0 + s) * ORC_NB, *y1i = yi + (o0 + s) * ORC_NB;
        double *y2r = yr + (o0 + 2 * (size_t)s) * ORC_NB, *y2i = yi + (o0 + 2 * (size_t)s) * ORC_NB;
        double *y3r = yr + (o0 + 3 * (size_t)s) * ORC_NB, *y3i = yi + (o0 + 3 * (size_t)s) * ORC_NB;
        const int k1 = pp * s * ts, k2 = 2 * k1, k3 = 3 * k1;
        const double w1r = P->wr[k1], w1i = sg * P->wi[k1], w2r = P->wr[k2], w2i = sg * P->wi[k2];
        const double w3r = P->wr[k3], w3i = sg * P->wi[k3];
        for (l = 0; l < ORC_NB; l++) {
          const double t0r = a0r[l] + a2r[l], t0i = a0i[l] + a2i[l];
          const double t1r = a0r[l] - a2r[l], t1i = a0i[l] - a2i[l];
          const double t2r = a1r[l] + a3r[l], t2i = a1i[l] + a3i[l];
          const double t3r = a1r[l] - a3r[l], t3i = a1i[l] - a3i[l];
          /* b1 = t1 + sign i t3, b3 = t1 - sign i t3 */
          const double b1r = t1r - sign * t3i, b1i = t1i + sign * t3r;
          const double b3r = t1r + sign * t3i, b3i = t1i - sign * t3r;
          const double b2r = t0r - t2r, b2i = t0i - t2i;
          y0r[l] = t0r + t2r;
          y0i[l] = t0i + t2i;
          y1r[l] = b1r * w1r - b1i * w1i;
          y1i[l] = b1r * w1i + b1i * w1r;
          y2r[l] = b2r * w2r - b2i * w2i;
          y2i[l] = b2r * w2i + b2i * w2r;
          y3r[l] = b3r * w3r - b3i * w3i;
          y3i[l] = b3r * w3i + b3i * w3r;
        }
      } else if (p == 2) {
        const double *a0r = xr + i0 * ORC_NB, *a0i = xi + i0 * ORC_NB;
        const double *a1r = xr + (i0 + (size_t)s * m) * ORC_NB, *a1i = xi + (i0 + (size_t)s * m) * ORC_NB;
        double *y0r = yr + o0 * ORC_NB, *y0i = yi + o0 * ORC_NB;
        double *y1r = yr + (o0 + s) * ORC_NB, *y1i = yi + (o0 + s) * ORC_NB;
        const int k1 = pp * s * ts;
        const double w1r = P->wr[k1], w1i = sg * P->wi[k1];
        for (l = 0; l < ORC_NB; l++) {
          const double br = a0r[l] - a1r[l], bi = a0i[l] - a1i[l];
          y0r[l] = a0r[l] + a1r[l];
          y0i[l] = a0i[l] + a1i[l];
          y1r[l] = br * w1r - bi * w1i;
          y1i[l] = br * w1i + bi * w1r;
        }
      } else if (p == 3) {
        const double c3 = -0.5, s3 = (double)(sign * 0.866025403784438646763723170752936183L);
        const double *a0r = xr + i0 * ORC_NB, *a0i = xi + i0 * ORC_NB;
        const double *a1r = xr + (i0 + (size_t)s * m) * ORC_NB, *a1i = xi + (i0 + (size_t)s * m) * ORC_NB;
        const double *a2r = xr + (i0 + (size_t)2 * s * m) * ORC_NB, *a2i = xi + (i0 + (size_t)2 * s * m) * ORC_NB;
        double *y0r = yr + o0 * ORC_NB, *y0i = yi + o0 * ORC_NB;
        double *y1r = yr + (o0 + s) * ORC_NB, *y1i = yi + (o0 + s) * ORC_NB;
        double *y2r = yr + (o0 + 2 * (size_t)s) * ORC_NB, *y2i = yi + (o0 + 2 * (size_t)s) * ORC_NB;
        const int k1 = pp * s * ts, k2 = 2 * k1;
        const double w1r = P->wr[k1], w1i = sg * P->wi[k1], w2r = P->wr[k2], w2i = sg * P->wi[k2];
        for (l = 0; l < ORC_NB; l++) {
          const double t1r = a1r[l] + a2r[l], t1i = a1i[l] + a2i[l];
          const double t2r = a1r[l] - a2r[l], t2i = a1i[l] - a2i[l];
          const double mr = a0r[l] + c3 * t1r, mi = a0i[l] + c3 * t1i;
          const double nr = -s3 * t2i, ni = s3 * t2r; /* i sign (sqrt3/2) t2 */
          const double b1r = mr + nr, b1i = mi + ni, b2r = mr - nr, b2i = mi - ni;
          y0r[l] = a0r[l] + t1r;
          y0i[l] = a0i[l] + t1i;
          y1r[l] = b1r * w1r - b1i * w1i;
          y1i[l] = b1r * w1i + b1i * w1r;
          y2r[l] = b2r * w2r - b2i * w2i;
          y2i[l] = b2r * w2i + b2i * w2r;
        }
      } else { /* direct DFT of length p */
        const int Np = N / p;
        for (t = 0; t < p; t++) {
          double *ytr = yr + (o0 + (size_t)t * s) * ORC_NB, *yti = yi + (o0 + (size_t)t * s) * ORC_NB;
          const int kt = t * pp * s * ts;
          const double wtr = P->wr[kt], wti = sg * P->wi[kt];
          double accr[ORC_NB], acci[ORC_NB];
          for (l = 0; l < ORC_NB; l++) accr[l] = acci[l] = 0.0;
          for (r = 0; r < p; r++) {
            const double *arr = xr + (i0 + (size_t)r * s * m) * ORC_NB, *ari = xi + (i0 + (size_t)r * s * m) * ORC_NB;
            const int kr = ((r * t) % p) * Np;
            const double cr = P->wr[kr], ci = sg * P->wi[kr];
            for (l = 0; l < ORC_NB; l++) {
              accr[l] += arr[l] * cr - ari[l] * ci;
              acci[l] += arr[l] * ci + ari[l] * cr;
            }
          }
          for (l = 0; l < ORC_NB; l++) {
            ytr[l] = accr[l] * wtr - acci[l] * wti;
            yti[l] = accr[l] * wti + acci[l] * wtr;
          }
        }
      }
    }
  }
}

/* FFT of length P->h of the B lines in (*xr, *xi), using (*yr, *yi) as the second buffer; on
 * return *xr / *xi point at the result. */
static void bfft(const bplan *P, int sign, double **xr, double **xi, double **yr, double **yi)
{
  int f, s = 1, m = P->h;
  for (f = 0; f < P->nf; f++) {
    const int p = P->fac[f];
    double *t;
    m /= p;
    bpass(P, p, m, s, sign, *xr, *xi, *yr, *yi);
    t = *xr; *xr = *yr; *yr = t;
    t = *xi; *xi = *yi; *yi = t;
    s *= p;
  }
}

/* compute_deriv_loc (deriv_line) on B lines of M complex values */
static void deriv_lines(double *xr, double *xi, int M, int r2c)
{
  int g = r2c ? (M - 1) * 2 : M, mid = g / 2, i, l;
  for (i = 0; i < M; i++) {
    double *pr = xr + (size_t)i * ORC_NB, *pi = xi + (size_t)i * ORC_NB;
    if (i == mid) {
      for (l = 0; l < ORC_NB; l++) pr[l] = pi[l] = 0.0;
      continue;
    }
    {
      const double k = (double)(i < mid ? i : i - g);
      for (l = 0; l < ORC_NB; l++) {
        const double re = pr[l], im = pi[l];
        pr[l] = -k * im;
        pi[l] = k * re;
      }
    }
  }
}

/* Whether a stage runs on the batched engine: C2C of any length, R2C / C2R of even length. */
static int batched_ok(int kind, int nlog)
{
  if (kind == ORC_K_C2C_FWD || kind == ORC_K_C2C_BWD) return nlog >= 1;
  if (kind == ORC_K_R2C || kind == ORC_K_C2R) return nlog >= 2 && nlog % 2 == 0;
  return 0;
}

static void exec_stage_batched(int kind, int dt1, int dt2, int nin, int nout, int nlog, const long long s1[3],
                               const long long s2[3], int L, int u, int v, long long nu, long long line0,
                               long long lend, const double *in, double *out, int deriv, int nthreads)
{
  const int half = (kind == ORC_K_R2C || kind == ORC_K_C2R);
  const int h = half ? nlog / 2 : nlog;
  bplan P;
  const long long nblk = (lend - line0 + ORC_NB - 1) / ORC_NB;
  bplan_init(&P, h, half ? 2 : 1);
#pragma omp parallel num_threads(nthreads)
  {
    const size_t cap = (size_t)((nin > nout ? nin : nout) + 2) * ORC_NB;
    double *buf = (double *)malloc(sizeof(double) * 4 * cap);
    long long blk;
#pragma omp for schedule(static)
    for (blk = 0; blk < nblk; blk++) {
      double *xr = buf, *xi = buf + cap, *yr = buf + 2 * cap, *yi = buf + 3 * cap;
      long long o1[ORC_NB], o2[ORC_NB];
      const long long l0 = line0 + blk * ORC_NB;
      const int nl = (int)(lend - l0 < ORC_NB ? lend - l0 : ORC_NB);
      int l, j, k;
      for (l = 0; l < ORC_NB; l++) {
        const long long ln = l0 + (l < nl ? l : 0), iu = ln % nu, iv = ln / nu;
        o1[l] = iu * s1[u] + iv * s1[v];
        o2[l] = iu * s2[u] + iv * s2[v];
      }
      /* gather */
      if (kind == ORC_K_R2C) {
        for (j = 0; j < h; j++)
          for (l = 0; l < ORC_NB; l++) {
            xr[(size_t)j * ORC_NB + l] = in[o1[l] + (2 * j) * s1[L]];
            xi[(size_t)j * ORC_NB + l] = in[o1[l] + (2 * j + 1) * s1[L]];
          }
      } else {
        for (j = 0; j < nin; j++)
          for (l = 0; l < ORC_NB; l++) {
            xr[(size_t)j * ORC_NB + l] = in[2 * (o1[l] + j * s1[L])];
            xi[(size_t)j * ORC_NB + l] = in[2 * (o1[l] + j * s1[L]) + 1];
          }
      }
      if (kind == ORC_K_C2C_FWD || kind == ORC_K_C2C_BWD) {
        bfft(&P, kind == ORC_K_C2C_FWD ? -1 : 1, &xr, &xi, &yr, &yi);
      } else if (kind == ORC_K_R2C) {
        /* Z = FFT_h(x[2m] + i x[2m+1]); X[k] = (Z[k] + conj Z[h-k]) / 2 - (i / 2) W^k (Z[k] - conj Z[h-k]) */
        bfft(&P, -1, &xr, &xi, &yr, &yi);
        for (k = 0; k <= h; k++) {
          const double *ar = xr + (size_t)(k % h) * ORC_NB, *ai = xi + (size_t)(k % h) * ORC_NB;
          const double *cr = xr + (size_t)((h - k) % h) * ORC_NB, *ci = xi + (size_t)((h - k) % h) * ORC_NB;
          double *Xr = yr + (size_t)k * ORC_NB, *Xi = yi + (size_t)k * ORC_NB;
          const double wr = P.wr[k], wi = P.wi[k];
          for (l = 0; l < ORC_NB; l++) {
            const double fer = 0.5 * (ar[l] + cr[l]), fei = 0.5 * (ai[l] - ci[l]);
            const double dr = ar[l] - cr[l], di = ai[l] + ci[l];
            const double for_ = 0.5 * di, foi = -0.5 * dr;
            Xr[l] = fer + (for_ * wr - foi * wi);
            Xi[l] = fei + (for_ * wi + foi * wr);
          }
        }
        { double *t = xr; xr = yr; yr = t; t = xi; xi = yi; yi = t; }
      } else { /* C2R: Z[k] = (X[k] + conj X[h-k]) + i W^-k (X[k] - conj X[h-k]); z = IFFT_h(Z) */
        for (l = 0; l < ORC_NB; l++) {
          xi[l] = 0.0;                   /* imag of DC ignored */
          xi[(size_t)h * ORC_NB + l] = 0.0; /* imag of Nyquist ignored */
        }
        for (k = 0; k < h; k++) {
          const double *ar = xr + (size_t)k * ORC_NB, *ai = xi + (size_t)k * ORC_NB;
          const double *cr = xr + (size_t)(h - k) * ORC_NB, *ci = xi + (size_t)(h - k) * ORC_NB;
          double *Zr = yr + (size_t)k * ORC_NB, *Zi = yi + (size_t)k * ORC_NB;
          const double wr = P.wr[k], wi = -P.wi[k]; /* exp(+2 pi i k / n) */
          for (l = 0; l < ORC_NB; l++) {
            const double fer = ar[l] + cr[l], fei = ai[l] - ci[l];
            const double dr = ar[l] - cr[l], di = ai[l] + ci[l];
            const double for_ = dr * wr - di * wi, foi = dr * wi + di * wr;
            Zr[l] = fer - foi;
            Zi[l] = fei + for_;
          }
        }
        { double *t = xr; xr = yr; yr = t; t = xi; xi = yi; yi = t; }
        bfft(&P, 1, &xr, &xi, &yr, &yi);
      }
      if (deriv && dt2 == 2) deriv_lines(xr, xi, nout, kind == ORC_K_R2C);
      /* scatter */
      if (kind == ORC_K_C2R) {
        for (j = 0; j < h; j++)
          for (l = 0; l < nl; l++) {
            out[o2[l] + (2 * j) * s2[L]] = xr[(size_t)j * ORC_NB + l];
            out[o2[l] + (2 * j + 1) * s2[L]] = xi[(size_t)j * ORC_NB + l];
          }
      } else {
        for (j = 0; j < nout; j++)
          for (l = 0; l < nl; l++) {
            out[2 * (o2[l] + j * s2[L])] = xr[(size_t)j * ORC_NB + l];
            out[2 * (o2[l] + j * s2[L]) + 1] = xi[(size_t)j * ORC_NB + l];
          }
      }
    }
    free(buf);
  }
  (void)dt1;
  bplan_free(&P);
}

/* ------------------------------------------------------------------------------------------ */
/* Planner, build/templ.C. */

/* swap0, templ.C:816-858: next memory order that makes dim L stride-1. */
void orc_swap0(int newmo[3], const int mo[3], int L)
{
  int i, j, tmp[3];
  for (i = 0; i < 3; i++) tmp[i] = mo[i];
  if (tmp[L] == 1) {
    for (j = 0; j < 3; j++)
      if (tmp[j] == 0) break;
    tmp[j] = 1;
    tmp[L] = 0;
  } else if (tmp[L] == 2) {
    for (i = 0; i < 3; i++) tmp[i] = (tmp[i] + 1) % 3;
  }
  for (i = 0; i < 3; i++) newmo[i] = tmp[i];
}

/* excl, templ.C:872-882 */
static int excl(int a, int b)
{
  if (a * b == 0) return ((a > b ? a : b) == 1) ? 2 : 1;
  return 0;
}

static int find_zero(const int a[3])
{
  int i;
  for (i = 0; i < 3; i++)
    if (a[i] == 0) return i;
  return -1;
}

/* find_order, templ.C:627-802, for one task on a 1x1x1 processor grid: Pdims == 1 for every
 * dim, ProcGrid::nd == 1 (init.C:1634-1641) and DataGrid::L = {0,1,2} (init.C:1813-1818). */
int orc_find_order(const int types[3], const orc_grid *g1, const orc_grid *g2, int L[3])
{
  int i, err = 0;
  orc_type_info ti;
  L[0] = L[1] = L[2] = -1;
  for (i = 0; i < 3; i++) {
    if (orc_type_info_get(types[i], &ti)) return -1;
    if (ti.dt1 < ti.dt2) {
      if (L[0] >= 0) err = 1; /* more than one R2C (templ.C:643-646) */
      else L[0] = i;
    } else if (ti.dt1 > ti.dt2) {
      if (L[2] >= 0) err = 1;
      else L[2] = i;
    }
  }
  if (L[0] >= 0 && L[2] >= 0) err = 1; /* templ.C:657-658 */
  if (L[0] < 0) {
    if (L[2] < 0) { /* templ.C:662-667 */
      L[0] = 0;
      if (g1->mo[0] > g1->mo[1]) L[0] = 1;
    } else { /* nd == 1 branch, templ.C:669-673 */
      L[0] = 0;
      if (L[0] == L[2]) L[0] = 1;
    }
  }
  if (L[2] < 0) { /* numtasks == 1, templ.C:692-697 */
    L[2] = find_zero(g2->mo);
    if (L[2] == L[0]) L[2] = (L[0] + 1) % 3;
  }
  L[1] = excl(L[0], L[2]); /* templ.C:792 */
  return err;
}

long long orc_grid_elems(const orc_grid *g)
{
  return (long long)g->gdims[0] * g->gdims[1] * g->gdims[2];
}

/* transform3D ctor stage loop, templ.C:224-420 (TRANS_ONLY branch: d1 stays -1 on one task). */
int orc_plan3d_make(const int types[3], const orc_grid *g1, const orc_grid *g2, orc_plan3d *p)
{
  int st, i, monext[3], mocurr[3], gd[3], dcs, err, dt_prev;
  orc_type_info ti;
  memset(p, 0, sizeof(*p));
  err = orc_find_order(types, g1, g2, p->L);
  if (err < 0) return -1;
  if (orc_type_info_get(types[p->L[0]], &ti)) return -1;
  p->dt1 = ti.dt1;
  p->prec = ti.prec;
  dt_prev = ti.dt1;
  for (i = 0; i < 3; i++) {
    monext[i] = g1->mo[i];
    gd[i] = g1->gdims[i];
  }
  dcs = g1->dcs;
  for (st = 0; st < 3; st++) {
    orc_stage *s = &p->st[p->nstages++];
    int Ls = p->L[st];
    for (i = 0; i < 3; i++) mocurr[i] = monext[i];
    if (orc_type_info_get(types[Ls], &ti)) return -1;
    if (ti.dt1 != dt_prev) err = 1; /* templ.C:296-297 */
    s->type = types[Ls];
    s->dim = Ls;
    for (i = 0; i < 3; i++) {
      s->g1.gdims[i] = gd[i];
      s->g1.mo[i] = mocurr[i];
    }
    s->g1.dcs = dcs;
    if (ti.dt1 < ti.dt2) { /* R2C, templ.C:270-273 */
      dcs = Ls;
      gd[dcs] = gd[dcs] / 2 + 1;
    } else if (ti.dt2 < ti.dt1) { /* C2R, templ.C:274-277 */
      if (dcs < 0 || dcs > 2) return -1;
      gd[dcs] = (gd[dcs] - 1) * 2;
      dcs = -1;
    }
    if (st < 2) { /* templ.C:279-285 */
      if (ti.kind != ORC_K_EMPTY) orc_swap0(monext, mocurr, Ls);
    } else { /* templ.C:287-291 */
      for (i = 0; i < 3; i++) monext[i] = g2->mo[i];
      if (monext[Ls] != 0) orc_swap0(monext, mocurr, Ls);
    }
    for (i = 0; i < 3; i++) {
      s->g2.gdims[i] = gd[i];
      s->g2.mo[i] = monext[i];
    }
    s->g2.dcs = dcs;
    dt_prev = ti.dt2;
  }
  p->dt2 = dt_prev;
  /* final_seq, templ.C:400-408 and 422-435 */
  if (monext[0] != g2->mo[0] || monext[1] != g2->mo[1] || monext[2] != g2->mo[2]) {
    orc_stage *s = &p->st[p->nstages++];
    int td = 0; /* grid2.L[0] */
    const orc_grid *prev = &p->st[p->nstages - 2].g2;
    if (prev->mo[td] != 0 && g2->mo[td] != 0) td = 1; /* grid2.nd == 1 on one task */
    s->type = (p->dt2 == 2) ? (p->prec == 4 ? 2 : 3) : (p->prec == 4 ? 0 : 1);
    s->dim = td;
    s->g1 = *prev;
    s->g2 = *g2;
  }
  for (i = 0; i < 3; i++)
    if (gd[i] != g2->gdims[i]) err = 1;
  p->ok = (err == 0);
  return err;
}

/* ------------------------------------------------------------------------------------------ */
/* Stage executor. */
static void strides_of(const orc_grid *g, long long s[3])
{
  int i, j;
  for (i = 0; i < 3; i++) {
    s[i] = 1;
    for (j = 0; j < 3; j++)
      if (g->mo[j] < g->mo[i]) s[i] *= g->gdims[j];
  }
}

int orc_exec_stage(const orc_stage *S, const double *in, double *out, int deriv, int nthreads)
{
  return orc_exec_stage_lines(S, in, out, deriv, nthreads, 0, -1);
}

int orc_exec_stage_lines(const orc_stage *S, const double *in, double *out, int deriv, int nthreads,
                         long long line0, long long line1)
{
  orc_type_info ti;
  int L = S->dim, a, b, nin, nout, nlog, kind;
  long long s1[3], s2[3], na, nb, line;
  lineplan LP;
  if (orc_type_info_get(S->type, &ti)) return -1;
  kind = ti.kind;
  a = (L + 1) % 3;
  b = (L + 2) % 3;
  if (S->g1.gdims[a] != S->g2.gdims[a] || S->g1.gdims[b] != S->g2.gdims[b]) return -2;
  nin = S->g1.gdims[L];
  nout = S->g2.gdims[L];
  nlog = (kind == ORC_K_C2R) ? nout : nin; /* transplan::init_tr, templ.C:933-960 */
  /* an empty line (e.g. the reference's C2R output length 2(M-1) for M = 1, templ.C:274-277) */
  if (nin <= 0 || nout <= 0) return -3;
  if (kind == ORC_K_R2C && nout != nin / 2 + 1) return -3;
  if (kind == ORC_K_C2R && nin != nout / 2 + 1) return -3;
  if ((kind != ORC_K_R2C && kind != ORC_K_C2R) && nin != nout) return -3;
  strides_of(&S->g1, s1);
  strides_of(&S->g2, s2);
  na = S->g1.gdims[a];
  nb = S->g1.gdims[b];
  if (ti.dt2 != 2) deriv = 0; /* compute_deriv_loc only acts on complex output, exec.C:245-286 */
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  if (g_batched && batched_ok(kind, nlog)) {
    /* blocks of lines neighbouring along the faster of the two other dims of the input */
    const int fast_b = s1[b] < s1[a];
    const long long lend = (line1 < 0 || line1 > na * nb) ? na * nb : line1;
    exec_stage_batched(kind, ti.dt1, ti.dt2, nin, nout, nlog, s1, s2, L, fast_b ? b : a, fast_b ? a : b,
                       fast_b ? nb : na, line0, lend, in, out, deriv, nthreads);
    return 0;
  }
  lineplan_init(&LP, kind, ti.r2r, nlog);
#pragma omp parallel num_threads(nthreads)
  {
    int maxn = (nin > nout ? nin : nout) + 2;
    int maxp = (kind != ORC_K_EMPTY && kind != ORC_K_R2R) ? LP.P.maxp : 1;
    double *lin = (double *)malloc(sizeof(double) * 2 * maxn);
    double *lout = (double *)malloc(sizeof(double) * 2 * maxn);
    double *work = (double *)malloc(sizeof(double) * (4 * (size_t)maxn + 2 * maxp + 8));
    long long ln;
    long long lend = (line1 < 0 || line1 > na * nb) ? na * nb : line1;
#pragma omp for schedule(static)
    for (ln = line0; ln < lend; ln++) {
      long long ia = ln % na, ib = ln / na, j;
      long long o1 = ia * s1[a] + ib * s1[b], o2 = ia * s2[a] + ib * s2[b];
      if (ti.dt1 == 2)
        for (j = 0; j < nin; j++) {
          lin[2 * j] = in[2 * (o1 + j * s1[L])];
          lin[2 * j + 1] = in[2 * (o1 + j * s1[L]) + 1];
        }
      else
        for (j = 0; j < nin; j++) lin[j] = in[o1 + j * s1[L]];
      switch (kind) {
        case ORC_K_EMPTY:
          memcpy(lout, lin, sizeof(double) * ti.dt1 * nin);
          break;
        case ORC_K_R2C: r2c_line(&LP, lin, lout, work); break;
        case ORC_K_C2R: c2r_line(&LP, lin, lout, work); break;
        case ORC_K_C2C_FWD: fft_exec(&LP.P, -1, lin, lout, work); break;
        case ORC_K_C2C_BWD: fft_exec(&LP.P, +1, lin, lout, work); break;
        case ORC_K_R2R:
          if (ti.dt1 == 2) {
            r2r_line(&LP, lin, 2, lout, 2);
            r2r_line(&LP, lin + 1, 2, lout + 1, 2);
          } else
            r2r_line(&LP, lin, 1, lout, 1);
          break;
      }
      if (deriv) deriv_line(lout, nout, kind == ORC_K_R2C);
      if (ti.dt2 == 2)
        for (j = 0; j < nout; j++) {
          out[2 * (o2 + j * s2[L])] = lout[2 * j];
          out[2 * (o2 + j * s2[L]) + 1] = lout[2 * j + 1];
        }
      else
        for (j = 0; j < nout; j++) out[o2 + j * s2[L]] = lout[j];
    }
    free(lin);
    free(lout);
    free(work);
  }
  (void)line;
  lineplan_free(&LP);
  return 0;
}

int orc_exec3d(const orc_plan3d *p, const double *in, double *out, int idir, int nthreads)
{
  int s, rc = 0;
  const double *cur = in;
  double *bufs[2] = {NULL, NULL};
  for (s = 0; s < p->nstages; s++) {
    const orc_stage *S = &p->st[s];
    orc_type_info ti;
    double *dst;
    orc_type_info_get(S->type, &ti);
    if (s == p->nstages - 1) dst = out;
    else {
      size_t sz = (size_t)orc_grid_elems(&S->g2) * ti.dt2;
      free(bufs[s & 1]);
      bufs[s & 1] = (double *)malloc(sizeof(double) * sz);
      dst = bufs[s & 1];
    }
    /* exec.C:175-178: the derivative is taken in the stage whose trans_dim == idir */
    rc = orc_exec_stage(S, cur, dst, (idir >= 0 && S->dim == idir && ti.kind != ORC_K_EMPTY), nthreads);
    if (rc) break;
    cur = dst;
  }
  free(bufs[0]);
  free(bufs[1]);
  return rc;
}

/* compute_deriv, build/deriv.C:85-184, on one task (GlobStart = 0).
 * ref_axis = 1 restates the reference literally: deriv.C:89-93 takes ldir with
 * MemOrder[ldir] == idir and then uses ldir as the STORAGE axis (deriv.C:107-180), i.e. it
 * differentiates along the storage axis holding the logical dim whose storage rank is idir, with
 * the wavenumbers of logical dim idir (g, mid from Gdims[idir], deriv.C:95-102).  For the identity
 * and transposition memory orders that is the storage axis of dim idir; for the 3-cycles (1,2,0)
 * and (2,0,1) it is another axis (QUIRK).  ref_axis = 0 differentiates along logical dim idir. */
int orc_compute_deriv_axis(const orc_grid *g, const double *in, double *out, int idir, int ref_axis)
{
  long long s[3], n0, n1, i, j;
  int a, b, gg, mid, M, ax = idir;
  if (idir < 0 || idir > 2) return -1;
  strides_of(g, s);
  if (ref_axis) {
    int d, ldir = idir;
    for (d = 0; d < 3; d++)
      if (g->mo[d] == idir) ldir = d; /* deriv.C:89-93 */
    for (d = 0; d < 3; d++)
      if (g->mo[d] == ldir) ax = d;   /* the logical dim stored at storage rank ldir */
  }
  M = g->gdims[ax];
  gg = (g->dcs == idir) ? (g->gdims[idir] - 1) * 2 : g->gdims[idir];
  mid = gg / 2;
  a = (ax + 1) % 3;
  b = (ax + 2) % 3;
  n0 = g->gdims[a];
  n1 = g->gdims[b];
  for (j = 0; j < n1; j++)
    for (i = 0; i < n0; i++) {
      int k;
      long long base = i * s[a] + j * s[b];
      for (k = 0; k < M; k++) {
        long long o = 2 * (base + (long long)k * s[ax]);
        double re = in[o], im = in[o + 1], kk;
        if (k < mid) kk = k;
        else if (k == mid) { out[o] = 0.0; out[o + 1] = 0.0; continue; }
        else kk = k - gg;
        out[o] = -kk * im;
        out[o + 1] = kk * re;
      }
    }
  return 0;
}

int orc_compute_deriv(const orc_grid *g, const double *in, double *out, int idir)
{
  return orc_compute_deriv_axis(g, in, out, idir, 0);
}
