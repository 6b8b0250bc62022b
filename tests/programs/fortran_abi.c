/*
 * The Fortran interface as a compiled Fortran program sees it, written in C (no Fortran compiler
 * is needed to run it).
 *
 * A Fortran program that uses the reference's module (build/fp3dfft++mod.f90) calls the *_f entry
 * points of include/Fwrap.h (reference build/wrap.C:575-792) with every argument by reference,
 * integer grid / type / plan handles and a 1-based derivative direction, and owns the type-ID
 * variables: the module's bind(C) variables (fp3dfft++mod.f90:8-24) are definitions in the program,
 * which p3dfft_setup fills in through the shared library's references.  This program does the
 * same:
 *   1. defines those 17 type-ID variables itself and checks that p3dfft_setup sets them to the
 *      reference's IDs (P3DFFT_EMPTY_TYPE, which no setup assigns, stays 0, as in the reference);
 *   2. (unless run with "ids") calls every *_f entry point and the matching C entry point on the
 *      same inputs and requires bit-identical outputs: 3D transforms and derivatives in double and
 *      single precision, 1D transforms, compute_deriv, and the grid queries.
 * Prints "Results are correct" and exits 0 when every check passes.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "p3dfft.h"

/* the module's variables, defined by the program */
int P3DFFT_EMPTY_TYPE;
int P3DFFT_R2CFFT_S, P3DFFT_R2CFFT_D, P3DFFT_C2RFFT_S, P3DFFT_C2RFFT_D;
int P3DFFT_CFFT_FORWARD_S, P3DFFT_CFFT_FORWARD_D, P3DFFT_CFFT_BACKWARD_S, P3DFFT_CFFT_BACKWARD_D;
int P3DFFT_DCT1_REAL_S, P3DFFT_DCT1_REAL_D, P3DFFT_DST1_REAL_S, P3DFFT_DST1_REAL_D;
int P3DFFT_DCT1_COMPLEX_S, P3DFFT_DCT1_COMPLEX_D, P3DFFT_DST1_COMPLEX_S, P3DFFT_DST1_COMPLEX_D;

static int failures = 0;

static void check(int ok, const char *what) {
  if (!ok) {
    printf("FAILED: %s\n", what);
    failures++;
  }
}

static void fill(double *a, long n, unsigned seed) {
  for (long i = 0; i < n; i++) {
    seed = seed * 1664525u + 1013904223u;
    a[i] = (double)(seed >> 8) / (double)(1u << 24) * 2.0 - 1.0;
  }
}

int main(int argc, char **argv) {
  const int want[17] = {0, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 16, 17, 14, 15, 18, 19};
  int i;
  MPI_Init(&argc, &argv);
  p3dfft_setup();
  {
    const int got[17] = {P3DFFT_EMPTY_TYPE, P3DFFT_R2CFFT_S, P3DFFT_R2CFFT_D, P3DFFT_C2RFFT_S, P3DFFT_C2RFFT_D,
                         P3DFFT_CFFT_FORWARD_S, P3DFFT_CFFT_FORWARD_D, P3DFFT_CFFT_BACKWARD_S, P3DFFT_CFFT_BACKWARD_D,
                         P3DFFT_DCT1_REAL_S, P3DFFT_DCT1_REAL_D, P3DFFT_DST1_REAL_S, P3DFFT_DST1_REAL_D,
                         P3DFFT_DCT1_COMPLEX_S, P3DFFT_DCT1_COMPLEX_D, P3DFFT_DST1_COMPLEX_S, P3DFFT_DST1_COMPLEX_D};
    for (i = 0; i < 17; i++) {
      char msg[64];
      snprintf(msg, sizeof msg, "type-ID variable %d = %d, expected %d", i, got[i], want[i]);
      check(got[i] == want[i], msg);
    }
  }
  if (argc > 1 && strcmp(argv[1], "ids") == 0) {
    printf(failures ? "Results are incorrect\n" : "Results are correct\n");
    return failures ? 1 : 0;
  }

  int pdims[3] = {1, 1, 1}, fcomm = MPI_Comm_c2f(MPI_COMM_WORLD);
  int gdims[3] = {32, 24, 20}, gdims2[3] = {17, 24, 20}, dmap[3] = {0, 1, 2};
  int mo1[3] = {0, 1, 2}, mo2[3] = {1, 2, 0}, dcs_none = -1, dcs_x = 0;
  int fpg = p3dfft_init_proc_grid_f(pdims, &fcomm);
  int cpg = p3dfft_init_proc_grid(pdims, MPI_COMM_WORLD);
  int fg1, fg2, ld[3], gs[3];
  p3dfft_init_data_grid_f(&fg1, ld, gs, gdims, &dcs_none, &fpg, dmap, mo1);
  check(ld[0] == 32 && ld[1] == 24 && ld[2] == 20 && gs[0] == 0 && gs[1] == 0 && gs[2] == 0,
        "init_data_grid_f local dims / global start");
  p3dfft_init_data_grid_f(&fg2, ld, gs, gdims2, &dcs_x, &fpg, dmap, mo2);
  check(ld[0] == 17, "init_data_grid_f conjugate-symmetric dims");
  Grid *cg1 = p3dfft_init_data_grid(gdims, -1, cpg, dmap, mo1);
  Grid *cg2 = p3dfft_init_data_grid(gdims2, 0, cpg, dmap, mo2);

  const long nr = 32L * 24 * 20, nc = 17L * 24 * 20;
  double *x = malloc(sizeof(double) * nr), *ya = malloc(16 * nc), *yb = malloc(16 * nc);
  double *za = malloc(sizeof(double) * nr), *zb = malloc(sizeof(double) * nr);
  float *xs = malloc(sizeof(float) * nr), *ysa = malloc(8 * nc), *ysb = malloc(8 * nc);
  fill(x, nr, 7u);
  for (long k = 0; k < nr; k++) xs[k] = (float)x[k];

  int prec, ow = 0;
  for (prec = 8; prec >= 4; prec -= 4) {
    int tf[3], tb[3], ftf, ftb, fpf, fpb;
    tf[0] = prec == 8 ? P3DFFT_R2CFFT_D : P3DFFT_R2CFFT_S;
    tf[1] = tf[2] = prec == 8 ? P3DFFT_CFFT_FORWARD_D : P3DFFT_CFFT_FORWARD_S;
    tb[0] = prec == 8 ? P3DFFT_C2RFFT_D : P3DFFT_C2RFFT_S;
    tb[1] = tb[2] = prec == 8 ? P3DFFT_CFFT_BACKWARD_D : P3DFFT_CFFT_BACKWARD_S;
    p3dfft_init_3Dtype_f(&ftf, tf);
    p3dfft_init_3Dtype_f(&ftb, tb);
    p3dfft_plan_3Dtrans_f(&fpf, &fg1, &fg2, &ftf);
    p3dfft_plan_3Dtrans_f(&fpb, &fg2, &fg1, &ftb);
    Plan3D cpf = p3dfft_plan_3Dtrans(cg1, cg2, p3dfft_init_3Dtype(tf));
    Plan3D cpb = p3dfft_plan_3Dtrans(cg2, cg1, p3dfft_init_3Dtype(tb));
    check(fpf >= 0 && fpb >= 0, "plan_3Dtrans_f");
    int idir;
    for (idir = 0; idir <= 3; idir++) {  /* 0: plain exec; 1..3: Fortran's 1-based direction */
      char msg[80];
      if (prec == 8) {
        if (idir == 0) {
          p3dfft_exec_3Dtrans_double_f(&fpf, x, ya, &ow);
          p3dfft_exec_3Dtrans_double(cpf, x, yb, 0);
        } else {
          p3dfft_exec_3Dderiv_double_f(&fpf, x, ya, &idir, &ow);
          p3dfft_exec_3Dderiv_double(cpf, x, yb, idir - 1, 0);
        }
        snprintf(msg, sizeof msg, "3D forward double, direction %d", idir);
        check(memcmp(ya, yb, 16 * nc) == 0, msg);
        p3dfft_exec_3Dtrans_double_f(&fpb, ya, za, &ow);
        p3dfft_exec_3Dtrans_double(cpb, ya, zb, 0);
        check(memcmp(za, zb, sizeof(double) * nr) == 0, "3D backward double");
      } else {
        if (idir == 0) {
          p3dfft_exec_3Dtrans_single_f(&fpf, xs, ysa, &ow);
          p3dfft_exec_3Dtrans_single(cpf, xs, ysb, 0);
        } else {
          p3dfft_exec_3Dderiv_single_f(&fpf, xs, ysa, &idir, &ow);
          p3dfft_exec_3Dderiv_single(cpf, xs, ysb, idir - 1, 0);
        }
        snprintf(msg, sizeof msg, "3D forward single, direction %d", idir);
        check(memcmp(ysa, ysb, 8 * nc) == 0, msg);
      }
    }
    /* a derivative really was taken along the 1-based direction: d/dz differs from d/dx */
    if (prec == 8) {
      int d1 = 1, d3 = 3;
      p3dfft_exec_3Dderiv_double_f(&fpf, x, ya, &d1, &ow);
      p3dfft_exec_3Dderiv_double_f(&fpf, x, yb, &d3, &ow);
      check(memcmp(ya, yb, 16 * nc) != 0, "derivative directions 1 and 3 differ");
    }
  }

  /* 1D: R2C along x from (0,1,2) to (1,2,0), double and single */
  for (prec = 8; prec >= 4; prec -= 4) {
    int t = prec == 8 ? P3DFFT_R2CFFT_D : P3DFFT_R2CFFT_S, dim = 0, fp1;
    p3dfft_plan_1Dtrans_f(&fp1, &fg1, &fg2, &t, &dim);
    int cp1 = p3dfft_plan_1Dtrans(cg1, cg2, t, 0);
    check(fp1 >= 0 && cp1 >= 0, "plan_1Dtrans_f");
    if (prec == 8) {
      p3dfft_exec_1Dtrans_double_f(&fp1, x, ya, &ow);
      p3dfft_exec_1Dtrans_double(cp1, x, yb, 0);
      check(memcmp(ya, yb, 16 * nc) == 0, "1D R2C double");
    } else {
      p3dfft_exec_1Dtrans_single_f(&fp1, xs, ysa, &ow);
      p3dfft_exec_1Dtrans_single(cp1, xs, ysb, 0);
      check(memcmp(ysa, ysb, 8 * nc) == 0, "1D R2C single");
    }
  }

  /* compute_deriv on the spectrum's grid, 1-based direction */
  {
    double *s = malloc(16 * nc);
    float *ss = malloc(8 * nc);
    fill(s, 2 * nc, 11u);
    for (long k = 0; k < 2 * nc; k++) ss[k] = (float)s[k];
    int idir;
    for (idir = 1; idir <= 3; idir++) {
      p3dfft_compute_deriv_double_f(s, ya, &fg2, &idir);
      p3dfft_compute_deriv_double(s, yb, cg2, idir - 1);
      check(memcmp(ya, yb, 16 * nc) == 0, "compute_deriv double");
      p3dfft_compute_deriv_single_f(ss, ysa, &fg2, &idir);
      p3dfft_compute_deriv_single(ss, ysb, cg2, idir - 1);
      check(memcmp(ysa, ysb, 8 * nc) == 0, "compute_deriv single");
    }
    free(s);
    free(ss);
  }
  check(p3dfft_last_error() == 0, "no error recorded");

  p3dfft_free_data_grid(cg1);
  p3dfft_free_data_grid(cg2);
  p3dfft_cleanup();
  free(x); free(ya); free(yb); free(za); free(zb); free(xs); free(ysa); free(ysb);
  printf(failures ? "Results are incorrect\n" : "Results are correct\n");
  MPI_Finalize();
  return failures ? 1 : 0;
}
