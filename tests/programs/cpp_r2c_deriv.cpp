// Drop-in check through the C++ API (include/p3dfft.h), following the flow of the reference
// sample programs sample/C++/test3D_r2c.C and sample/C++/test_deriv.C on a 1x1x1 grid:
// forward R2C/C2C/C2C of sin*sin*sin, spectrum must be +-0.125i at (+-1,+-1,+-1) after 1/N^3;
// backward must recover the field; exec_deriv(idir) + backward must give cos in dim idir.
// Usage: cpp_r2c_deriv nx ny nz   (exit code 0 = correct)
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "p3dfft.h"

using namespace p3dfft;

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  int g[3] = {argc > 1 ? atoi(argv[1]) : 32, argc > 2 ? atoi(argv[2]) : 32, argc > 3 ? atoi(argv[3]) : 32};
  setup();
  int ids1[3] = {R2CFFT_D, CFFT_FORWARD_D, CFFT_FORWARD_D};
  int ids2[3] = {C2RFFT_D, CFFT_BACKWARD_D, CFFT_BACKWARD_D};
  trans_type3D type_rcc(ids1), type_ccr(ids2);
  int pdims[3] = {1, 1, 1}, mo1[3] = {0, 1, 2}, mo2[3] = {1, 2, 0}, dmap1[3] = {0, 1, 2}, dmap2[3] = {1, 2, 0};
  ProcGrid pgrid(pdims, MPI_COMM_WORLD);
  DataGrid X(g, -1, &pgrid, dmap1, mo1);
  int g2[3] = {g[0] / 2 + 1, g[1], g[2]};
  DataGrid Z(g2, 0, &pgrid, dmap2, mo2);
  transform3D<double, complex_double> fwd(X, Z, &type_rcc);
  transform3D<complex_double, double> bwd(Z, X, &type_ccr);
  long n1 = (long)X.Ldims[0] * X.Ldims[1] * X.Ldims[2];
  long n2 = (long)Z.Ldims[0] * Z.Ldims[1] * Z.Ldims[2];
  double *in = new double[n1], *fin = new double[n1];
  complex_double *out = new complex_double[n2];
  const double twopi = 8.0 * atan(1.0);
  for (int z = 0; z < g[2]; z++)
    for (int y = 0; y < g[1]; y++)
      for (int x = 0; x < g[0]; x++)
        in[x + g[0] * (y + (long)g[1] * z)] = sin(x * twopi / g[0]) * sin(y * twopi / g[1]) * sin(z * twopi / g[2]);
  fwd.exec(in, out, false);
  const double nglob = (double)g[0] * g[1] * g[2];
  double dmax = 0;
  // storage of Z: z fastest, then x (N/2+1), then y
  for (int y = 0; y < g2[1]; y++)
    for (int x = 0; x < g2[0]; x++)
      for (int z = 0; z < g2[2]; z++) {
        complex_double v = out[z + g2[2] * (x + (long)g2[0] * y)] / nglob, ans = 0.0;
        if (x == 1 && (y == 1 || y == g[1] - 1) && (z == 1 || z == g[2] - 1))
          ans = complex_double(0.0, 0.125 * (y == 1 ? 1 : -1) * (z == 1 ? 1 : -1));
        dmax = fmax(dmax, abs(v - ans));
        out[z + g2[2] * (x + (long)g2[0] * y)] = v;
      }
  int bad = dmax > 1e-14 * g[0] * 0.25;
  printf("forward max diff %g\n", dmax);
  bwd.exec(out, fin, true);
  double rmax = 0;
  for (long i = 0; i < n1; i++) rmax = fmax(rmax, fabs(fin[i] - in[i]));
  printf("round trip max diff %g\n", rmax);
  bad |= rmax > 1e-14 * nglob * 0.25;
  for (int idir = 0; idir < 3; idir++) {
    fwd.exec_deriv(in, out, idir, false);
    for (long i = 0; i < n2; i++) out[i] /= nglob;
    bwd.exec(out, fin, true);
    double m = 0;
    for (int z = 0; z < g[2]; z++)
      for (int y = 0; y < g[1]; y++)
        for (int x = 0; x < g[0]; x++) {
          double fx = idir == 0 ? cos(x * twopi / g[0]) : sin(x * twopi / g[0]);
          double fy = idir == 1 ? cos(y * twopi / g[1]) : sin(y * twopi / g[1]);
          double fz = idir == 2 ? cos(z * twopi / g[2]) : sin(z * twopi / g[2]);
          m = fmax(m, fabs(fin[x + g[0] * (y + (long)g[1] * z)] - fx * fy * fz));
        }
    printf("derivative idir=%d max diff %g\n", idir, m);
    bad |= m > 1e-14 * nglob * 0.25;
  }
  printf(bad ? "Results are incorrect\n" : "Results are correct\n");
  delete[] in;
  delete[] fin;
  delete[] out;
  cleanup();
  MPI_Finalize();
  return bad || p3dfft_last_error() != 0;
}
