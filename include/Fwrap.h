/*
 * Fortran-callable entry points of the GB300 P3DFFT++ pipeline (libp3dfft_gb300.so).
 *
 * Same symbols and by-reference argument conventions as the reference Fortran glue
 * (reference include/Fwrap.h:81-93, implemented in build/wrap.C:575-792; bound from Fortran by
 * build/fp3dfft++mod.f90).  Grids are integer handles into the library's grid table; `idir`
 * is 1-based (wrap.C:627, 774).
 *
 *   p3dfft_init_3Dtype_f            wrap.C:575-583
 *   p3dfft_plan_1Dtrans_f           wrap.C:585-619
 *   p3dfft_compute_deriv_*_f        wrap.C:621-634
 *   p3dfft_plan_3Dtrans_f           wrap.C:636-703
 *   p3dfft_init_proc_grid_f         wrap.C:705-710
 *   p3dfft_init_data_grid_f         wrap.C:712-752
 *   p3dfft_exec_3Dtrans_*_f         wrap.C:755-763
 *   p3dfft_exec_3Dderiv_*_f         wrap.C:764-772
 *   p3dfft_exec_1Dtrans_*_f         wrap.C:775-783
 */
#ifndef P3DFFT_GB300_FWRAP_H
#define P3DFFT_GB300_FWRAP_H

void p3dfft_init_3Dtype_f(int *, int[3]);
void p3dfft_plan_1Dtrans_f(int *, int *, int *, int *, int *);
void p3dfft_plan_3Dtrans_f(int *, int *, int *, Type3D *);
int p3dfft_init_proc_grid_f(int *pdims, int *mpicomm);
void p3dfft_init_data_grid_f(int *mygrid, int *ldims, int *glob_start, int *gdims, int *dim_conj_sym,
                             int *pgrid_id, int *dmap, int *mem_order);
void p3dfft_exec_1Dtrans_double_f(int *, double *, double *, int *);
void p3dfft_exec_1Dtrans_single_f(int *, float *, float *, int *);
void p3dfft_exec_3Dtrans_double_f(Plan3D *, double *, double *, int *);
void p3dfft_exec_3Dtrans_single_f(Plan3D *, float *, float *, int *);
void p3dfft_exec_3Dderiv_double_f(Plan3D *, double *, double *, int *, int *);
void p3dfft_exec_3Dderiv_single_f(Plan3D *, float *, float *, int *, int *);
void p3dfft_compute_deriv_single_f(float *, float *, int *, int *);
void p3dfft_compute_deriv_double_f(double *, double *, int *, int *);

#endif
