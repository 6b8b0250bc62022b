/*
 * C interface of the GB300 P3DFFT++ transform pipeline (libp3dfft_gb300.so).
 *
 * Same declarations, argument meaning and struct layout as the reference C wrappers
 * (reference include/Cwrap.h:80-121, implemented in build/wrap.C:85-571).  Included by
 * p3dfft.h inside extern "C".  Data pointers may be host memory (pageable or pinned; the
 * library stages it through HBM) or device memory (used in place).
 *
 * Entry points and the reference interface each one replaces:
 *   p3dfft_setup / p3dfft_cleanup            wrap.C:90-141        (init.C:121 setup, cleanup)
 *   p3dfft_init_3Dtype                       wrap.C:148-154       (trans_type3D ctor init.C:2027)
 *   p3dfft_plan_1Dtrans                      wrap.C:236-279       (transplan ctor templ.C:994)
 *   p3dfft_plan_3Dtrans                      wrap.C:157-232       (transform3D ctor templ.C:91)
 *   find_grid                                wrap.C:281-297
 *   p3dfft_init_proc_grid                    wrap.C:299-304       (ProcGrid ctor init.C:1631)
 *   p3dfft_init_data_grid                    wrap.C:307-327       (DataGrid ctor init.C:1699)
 *   p3dfft_free_data_grid/_proc_grid         wrap.C:336-346
 *   p3dfft_inv_mo                            wrap.C:348-350       (inv_mo exec.C:2959)
 *   p3dfft_exec_1Dtrans_double/_single       wrap.C:483-549       (transplan::exec exec.C:522)
 *   p3dfft_exec_3Dtrans_double/_single       wrap.C:357-417       (transform3D::exec exec.C:290)
 *   p3dfft_exec_3Dderiv_double/_single       wrap.C:419-481       (transform3D::exec_deriv exec.C:101)
 *   p3dfft_compute_deriv_single/_double      wrap.C:551-568       (compute_deriv deriv.C:85)
 */
#ifndef P3DFFT_GB300_CWRAP_H
#define P3DFFT_GB300_CWRAP_H

struct CDataGrid_struct {
  int nd;           /* number of dimensions the volume is split over */
  int Gdims[3];     /* global dimensions */
  int dim_conj_sym; /* dimension holding N/2+1 after an R2C transform, -1 if none */
  int MemOrder[3];  /* storage rank of each logical dimension, 0 = stride-1 */
  int Ldims[3];     /* local dimensions (= Gdims on one rank) */
  int Dmap[3];      /* data dimension -> processor grid dimension */
  int pgrid;        /* processor grid handle */
  int grid_id[3];   /* position in the processor grid */
  int GlobStart[3]; /* start of the local block in the global grid */
  int taskid, numtasks;
  int ProcDims[3];
  MPI_Comm mpi_comm_glob;
};

typedef struct CDataGrid_struct CDataGrid;
typedef struct CDataGrid_struct Grid;

void p3dfft_setup();
void p3dfft_cleanup();
Type3D p3dfft_init_3Dtype(int[3]);
int p3dfft_plan_1Dtrans(Grid *, Grid *, int, int);
Plan3D p3dfft_plan_3Dtrans(Grid *, Grid *, Type3D);
int find_grid(int[3], int, int *, int[3]);
int p3dfft_init_proc_grid(int pdims[3], MPI_Comm comm);
Grid *p3dfft_init_data_grid(int[3], int, int, int[3], int[3]);
void p3dfft_free_data_grid(Grid *gr);
void p3dfft_free_proc_grid(int pgrid);
void p3dfft_inv_mo(int[3], int[3]);
void p3dfft_exec_1Dtrans_double(int, double *, double *, int);
void p3dfft_exec_1Dtrans_single(int, float *, float *, int);
void p3dfft_exec_3Dtrans_double(Plan3D, double *, double *, int);
void p3dfft_exec_3Dtrans_single(Plan3D, float *, float *, int);
void p3dfft_exec_3Dderiv_double(Plan3D, double *, double *, int, int);
void p3dfft_exec_3Dderiv_single(Plan3D, float *, float *, int, int);
void p3dfft_compute_deriv_single(float *, float *, Grid *, int);
void p3dfft_compute_deriv_double(double *, double *, Grid *, int);

#endif
