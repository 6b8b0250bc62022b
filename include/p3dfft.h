/*
 * p3dfft.h -- public header of the GB300-native P3DFFT++ 3D transform pipeline.
 *
 * Source-compatible with the reference header (reference include/p3dfft.h) for the calls a
 * P3DFFT++ program makes on a 1x1x1 processor grid: the type-ID globals (p3dfft.h:105-160),
 * setup()/cleanup(), ProcGrid (653-699), DataGrid (702-755), trans_type3D (832-849),
 * transform3D<T1,T2> (877-896), transplan<T1,T2> (581-623), compute_deriv<T> (917),
 * inv_mo, the timer class (958-992) and the C / Fortran wrappers (Cwrap.h, Fwrap.h).
 *
 * The templates are thin inline wrappers over the plain-C entry points of p3dfft_gb300.h, so the
 * library's exported interface is C-ABI only (ints and pointers).  Data arrays may live in host
 * memory (staged through HBM by the library) or in device memory (used in place).
 */
#ifndef P3DFFT_GB300_P3DFFT_H
#define P3DFFT_GB300_P3DFFT_H

#include "mpi.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define Type3D int
#define Type1D int
#define Plan3D int
#define Plan1D int

#ifdef __cplusplus
extern "C" {
#endif

extern int P3DFFT_EMPTY_TYPE_SINGLE, P3DFFT_EMPTY_TYPE_DOUBLE, P3DFFT_EMPTY_TYPE_SINGLE_COMPLEX,
    P3DFFT_EMPTY_TYPE_DOUBLE_COMPLEX;
extern int P3DFFT_R2CFFT_S, P3DFFT_R2CFFT_D, P3DFFT_C2RFFT_S, P3DFFT_C2RFFT_D, P3DFFT_CFFT_FORWARD_S,
    P3DFFT_CFFT_FORWARD_D, P3DFFT_CFFT_BACKWARD_S, P3DFFT_CFFT_BACKWARD_D;
extern int P3DFFT_DCT1_REAL_S, P3DFFT_DCT1_REAL_D, P3DFFT_DST1_REAL_S, P3DFFT_DST1_REAL_D,
    P3DFFT_DCT1_COMPLEX_S, P3DFFT_DCT1_COMPLEX_D, P3DFFT_DST1_COMPLEX_S, P3DFFT_DST1_COMPLEX_D;
extern int P3DFFT_DCT2_REAL_S, P3DFFT_DCT2_REAL_D, P3DFFT_DST2_REAL_S, P3DFFT_DST2_REAL_D,
    P3DFFT_DCT2_COMPLEX_S, P3DFFT_DCT2_COMPLEX_D, P3DFFT_DST2_COMPLEX_S, P3DFFT_DST2_COMPLEX_D;
extern int P3DFFT_DCT3_REAL_S, P3DFFT_DCT3_REAL_D, P3DFFT_DST3_REAL_S, P3DFFT_DST3_REAL_D,
    P3DFFT_DCT3_COMPLEX_S, P3DFFT_DCT3_COMPLEX_D, P3DFFT_DST3_COMPLEX_S, P3DFFT_DST3_COMPLEX_D;
extern int P3DFFT_DCT4_REAL_S, P3DFFT_DCT4_REAL_D, P3DFFT_DST4_REAL_S, P3DFFT_DST4_REAL_D,
    P3DFFT_DCT4_COMPLEX_S, P3DFFT_DCT4_COMPLEX_D, P3DFFT_DST4_COMPLEX_S, P3DFFT_DST4_COMPLEX_D;

#include "Cwrap.h"
#include "Fwrap.h"
#include "p3dfft_gb300.h"

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
#include <complex>
#include <iostream>
#include <typeinfo>
#include <vector>

namespace p3dfft {

using namespace std;

static const int REAL = 1;
static const int COMPLEX = 2;
static const int TRANS_ONLY = 1;
static const int MPI_ONLY = 2;
static const int TRANSMPI = 3;

extern int EMPTY_TYPE_SINGLE, EMPTY_TYPE_DOUBLE, EMPTY_TYPE_SINGLE_COMPLEX, EMPTY_TYPE_DOUBLE_COMPLEX;
extern int R2CFFT_S, R2CFFT_D, C2RFFT_S, C2RFFT_D, CFFT_FORWARD_S, CFFT_FORWARD_D, CFFT_BACKWARD_S,
    CFFT_BACKWARD_D;
extern int DCT1_REAL_S, DCT1_REAL_D, DST1_REAL_S, DST1_REAL_D, DCT1_COMPLEX_S, DCT1_COMPLEX_D, DST1_COMPLEX_S,
    DST1_COMPLEX_D;
extern int DCT2_REAL_S, DCT2_REAL_D, DST2_REAL_S, DST2_REAL_D, DCT2_COMPLEX_S, DCT2_COMPLEX_D, DST2_COMPLEX_S,
    DST2_COMPLEX_D;
extern int DCT3_REAL_S, DCT3_REAL_D, DST3_REAL_S, DST3_REAL_D, DCT3_COMPLEX_S, DCT3_COMPLEX_D, DST3_COMPLEX_S,
    DST3_COMPLEX_D;
extern int DCT4_REAL_S, DCT4_REAL_D, DST4_REAL_S, DST4_REAL_D, DCT4_COMPLEX_S, DCT4_COMPLEX_D, DST4_COMPLEX_S,
    DST4_COMPLEX_D;

typedef complex<float> mycomplex;
typedef complex<double> complex_double;

void setup();
void cleanup();
void inv_mo(int mo[3], int imo[3]);
void rel_change(int *, int *, int *);

class ProcGrid {
 public:
  int taskid, numtasks;
  int nd;
  int ProcDims[3];
  int grid_id_cart[3];
  MPI_Comm mpi_comm_glob;
  MPI_Comm mpi_comm_cart;
  MPI_Comm mpicomm[3];
  ProcGrid(int procdims[3], MPI_Comm mpi_comm_init);
  ProcGrid(const ProcGrid &rhs);
  ~ProcGrid();
  bool operator==(const ProcGrid &P) const;
};

class DataGrid {
 public:
  int nd;
  int Gdims[3];
  int dim_conj_sym;
  int MemOrder[3];
  int Ldims[3];
  ProcGrid *Pgrid;
  int Pdims[3];
  int Dmap[3];
  int L[3];
  int D[3];
  int GlobStart[3];
  int grid_id[3];
  bool is_set;
  inline bool IsLocal(int dim) {
    if (dim < 0 || dim > 2) return false;
    return Pdims[dim] == 1;
  }
  DataGrid(int *gdims_, int dim_conj_sym_, ProcGrid *pgrid, int *dmap, int *mem_order);
  DataGrid(const DataGrid &rhs);
  DataGrid() : is_set(false) {}
  ~DataGrid();
  void set_gdims(int gdims[3]);
  void get_gdims(int gdims[3]) {
    for (int i = 0; i < 3; i++) gdims[i] = Gdims[i];
  }
  void set_mo(int mo[3]) {
    for (int i = 0; i < 3; i++) MemOrder[i] = mo[i];
  }
};

class trans_type3D {
 public:
  char *name;
  int prec;
  bool is_set;
  int types[3];
  trans_type3D(int types_IDs[3]);
  trans_type3D(const trans_type3D &rhs);
  ~trans_type3D();
};

template <class T>
struct p3d_elem {};
template <>
struct p3d_elem<float> {
  enum { prec = 4, dt = 1 };
};
template <>
struct p3d_elem<double> {
  enum { prec = 8, dt = 1 };
};
template <>
struct p3d_elem<mycomplex> {
  enum { prec = 4, dt = 2 };
};
template <>
struct p3d_elem<complex_double> {
  enum { prec = 8, dt = 2 };
};

class gen_transform3D {
 public:
  int prec;
  int dt1, dt2;
  bool OW;
};

// 3D transform, planned by the constructor (reference templ.C:91-420) and executed by
// exec / exec_deriv (exec.C:101-295).
template <class Type1, class Type2>
class transform3D : public gen_transform3D {
  int handle_;

 public:
  bool is_set;
  transform3D(const DataGrid &grid1_, const DataGrid &grid2_, const trans_type3D *type) : handle_(-1), is_set(false) {
    prec = p3d_elem<Type1>::prec;
    dt1 = p3d_elem<Type1>::dt;
    dt2 = p3d_elem<Type2>::dt;
    OW = false;
    if ((int)p3d_elem<Type2>::prec != prec) cout << "Error in transform3D: precisions don't match!" << endl;
    handle_ = p3dfft_gb300_plan3d(type->types, grid1_.Gdims, grid1_.MemOrder, grid1_.dim_conj_sym, grid2_.Gdims,
                                  grid2_.MemOrder, grid2_.dim_conj_sym);
    if (handle_ < 0) {
      cout << "Error in transform3D: " << p3dfft_last_error_string() << endl;
      return;
    }
    int a, b, p;
    p3dfft_gb300_plan3d_types(handle_, &a, &b, &p);
    if (a != dt1) printf("Error in transform3D: input datatypes don't match\n");
    if (b != dt2) printf("Error in transform3D: output datatypes don't match\n");
    is_set = (a == dt1 && b == dt2 && p == prec);
  }
  ~transform3D() {
    if (handle_ >= 0) p3dfft_gb300_destroy3d(handle_);
  }
  void exec(Type1 *in, Type2 *out, bool OW_ = false) { p3dfft_gb300_exec3d(handle_, in, out, -1, OW_ ? 1 : 0); }
  void exec_deriv(Type1 *in, Type2 *out, int idir, bool OW_ = false) {
    p3dfft_gb300_exec3d(handle_, in, out, idir, OW_ ? 1 : 0);
  }
  int handle() const { return handle_; }

 private:
  transform3D(const transform3D &);
  transform3D &operator=(const transform3D &);
};

// One 1D transform combined with a local reorder (reference transplan, templ.C:900-1075,
// exec.C:522-702).
template <class Type1, class Type2>
class transplan {
  int handle_;

 public:
  int trans_dim;
  bool is_set;
  transplan(const DataGrid &gr1, const DataGrid &gr2, int type_ID, int d) : handle_(-1), trans_dim(d), is_set(false) {
    handle_ = p3dfft_gb300_plan1d(type_ID, gr1.Gdims, gr1.MemOrder, gr1.dim_conj_sym, gr2.Gdims, gr2.MemOrder,
                                  gr2.dim_conj_sym, d);
    if (handle_ < 0) {
      cout << "Error in transplan: " << p3dfft_last_error_string() << endl;
      return;
    }
    is_set = true;
  }
  ~transplan() {
    if (handle_ >= 0) p3dfft_gb300_destroy1d(handle_);
  }
  void exec(char *in, char *out, bool OW = false) { p3dfft_gb300_exec1d(handle_, in, out, OW ? 1 : 0); }
  int handle() const { return handle_; }

 private:
  transplan(const transplan &);
  transplan &operator=(const transplan &);
};

// Spectral derivative d/dx_idir of a complex field stored on grid *gr (reference deriv.C:85).
template <class Type>
void compute_deriv(Type *in, Type *out, DataGrid *gr, int idir) {
  p3dfft_gb300_compute_deriv(p3d_elem<Type>::prec, in, out, gr->Gdims, gr->MemOrder, gr->dim_conj_sym, idir);
}

// Per-phase timers (reference p3dfft.h:958-992); device time of each phase in seconds.
class timer {
 public:
  double reorder_deriv, reorder_trans, reorder_out, reorder_in, trans_exec, trans_deriv;
  double packsend, packsend_trans, packsend_deriv, unpackrecv, alltoall;
  void init();
  void print(MPI_Comm);
};
extern timer timers;

}  // namespace p3dfft

#endif  // __cplusplus
#endif
