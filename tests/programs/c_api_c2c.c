/* Drop-in check through the C API (include/Cwrap.h), following sample/C/test3D_c2c.c and
 * sample/C/test_deriv.c on a 1x1x1 grid: complex 3D forward / backward transforms in double and
 * single precision with memory orders (0,1,2) -> (2,1,0), plus p3dfft_compute_deriv_double.
 * Usage: c_api_c2c nx ny nz   (exit code 0 = correct) */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "p3dfft.h"

int main(int argc, char **argv) {
  int g[3], pdims[3] = {1, 1, 1}, mo1[3] = {0, 1, 2}, mo2[3] = {2, 1, 0}, dmap[3] = {0, 1, 2};
  int i, x, y, z, bad = 0;
  long n;
  MPI_Init(&argc, &argv);
  g[0] = argc > 1 ? atoi(argv[1]) : 16;
  g[1] = argc > 2 ? atoi(argv[2]) : 12;
  g[2] = argc > 3 ? atoi(argv[3]) : 10;
  n = (long)g[0] * g[1] * g[2];
  p3dfft_setup();
  int f_ids[3] = {P3DFFT_CFFT_FORWARD_D, P3DFFT_CFFT_FORWARD_D, P3DFFT_CFFT_FORWARD_D};
  int b_ids[3] = {P3DFFT_CFFT_BACKWARD_D, P3DFFT_CFFT_BACKWARD_D, P3DFFT_CFFT_BACKWARD_D};
  int fs_ids[3] = {P3DFFT_CFFT_FORWARD_S, P3DFFT_CFFT_FORWARD_S, P3DFFT_CFFT_FORWARD_S};
  Type3D tf = p3dfft_init_3Dtype(f_ids), tb = p3dfft_init_3Dtype(b_ids), tfs = p3dfft_init_3Dtype(fs_ids);
  int pg = p3dfft_init_proc_grid(pdims, MPI_COMM_WORLD);
  Grid *g1 = p3dfft_init_data_grid(g, -1, pg, dmap, mo1);
  Grid *g2 = p3dfft_init_data_grid(g, -1, pg, dmap, mo2);
  Plan3D pf = p3dfft_plan_3Dtrans(g1, g2, tf), pb = p3dfft_plan_3Dtrans(g2, g1, tb);
  Plan3D pfs = p3dfft_plan_3Dtrans(g1, g2, tfs);
  double *in = malloc(sizeof(double) * 2 * n), *out = malloc(sizeof(double) * 2 * n);
  double *fin = malloc(sizeof(double) * 2 * n);
  float *ins = malloc(sizeof(float) * 2 * n), *outs = malloc(sizeof(float) * 2 * n);
  const double twopi = 8.0 * atan(1.0);
  /* exp(2 pi i (x/Nx + 2y/Ny + 3z/Nz)) has one nonzero mode (1,2,3) of value Nx*Ny*Nz */
  for (z = 0; z < g[2]; z++)
    for (y = 0; y < g[1]; y++)
      for (x = 0; x < g[0]; x++) {
        long k = x + g[0] * (y + (long)g[1] * z);
        double ph = twopi * ((double)x / g[0] + 2.0 * y / g[1] + 3.0 * z / g[2]);
        in[2 * k] = cos(ph);
        in[2 * k + 1] = sin(ph);
        ins[2 * k] = (float)in[2 * k];
        ins[2 * k + 1] = (float)in[2 * k + 1];
      }
  p3dfft_exec_3Dtrans_double(pf, in, out, 0);
  p3dfft_exec_3Dtrans_single(pfs, ins, outs, 0);
  double dmax = 0, smax = 0;
  /* output memory order (2,1,0): x slowest, z fastest */
  for (x = 0; x < g[0]; x++)
    for (y = 0; y < g[1]; y++)
      for (z = 0; z < g[2]; z++) {
        long k = z + g[2] * (y + (long)g[1] * x);
        double ar = (x == 1 && y == 2 && z == 3) ? (double)n : 0.0;
        dmax = fmax(dmax, hypot(out[2 * k] / n - ar / n, out[2 * k + 1] / n));
        smax = fmax(smax, hypot(outs[2 * k] / n - ar / n, outs[2 * k + 1] / n));
      }
  printf("double forward max diff %g, single %g\n", dmax, smax);
  bad |= dmax > 1e-14 * g[0] * 0.25 || smax > 1e-6 * g[0];
  /* spectral derivative along y of the spectrum: i*k_y times it, k_y = 2 */
  p3dfft_compute_deriv_double(out, fin, g2, 1);
  long kk = 3 + g[2] * (2 + (long)g[1] * 1);
  double er = fabs(fin[2 * kk] - 0.0) + fabs(fin[2 * kk + 1] - 2.0 * n);
  printf("compute_deriv check %g\n", er / n);
  bad |= er / n > 1e-13;
  p3dfft_exec_3Dtrans_double(pb, out, fin, 1);
  double rmax = 0;
  for (i = 0; i < 2 * n; i++) rmax = fmax(rmax, fabs(fin[i] / n - in[i]));
  printf("round trip max diff %g\n", rmax);
  bad |= rmax > 1e-14 * n * 0.25;
  printf(bad ? "Results are incorrect\n" : "Results are correct\n");
  p3dfft_free_data_grid(g1);
  p3dfft_free_data_grid(g2);
  p3dfft_cleanup();
  MPI_Finalize();
  free(in); free(out); free(fin); free(ins); free(outs);
  return bad || p3dfft_last_error() != 0;
}
