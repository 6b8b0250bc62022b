/*
 * Single-rank MPI shim for P3DFFT++ programs run on one GPU (libp3dfft_mpi1.so).
 *
 * P3DFFT++'s public header includes "mpi.h" (reference include/p3dfft.h:87) and its sample
 * programs call a small set of MPI routines.  On a one-GPU, one-rank (1x1x1 processor grid)
 * run none of them communicates, so this header plus libp3dfft_mpi1.so provide exactly that set
 * with single-rank semantics: rank 0 of size 1, collectives copy send to receive buffers,
 * point-to-point calls are not supported.  Programs that link a real MPI do not use this file.
 */
#ifndef P3DFFT_GB300_MPI_SINGLE_H
#define P3DFFT_GB300_MPI_SINGLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#define MPI_COMM_SELF ((MPI_Comm)0x44000001)

/* datatypes: the low byte holds the element size in bytes */
#define MPI_CHAR ((MPI_Datatype)0x4c000101)
#define MPI_BYTE ((MPI_Datatype)0x4c00010d)
#define MPI_INT ((MPI_Datatype)0x4c000405)
#define MPI_LONG ((MPI_Datatype)0x4c000807)
#define MPI_FLOAT ((MPI_Datatype)0x4c00040a)
#define MPI_REAL ((MPI_Datatype)0x4c00041c)
#define MPI_DOUBLE ((MPI_Datatype)0x4c00080b)
#define MPI_DOUBLE_PRECISION ((MPI_Datatype)0x4c00081f)
#define MPI_COMPLEX ((MPI_Datatype)0x4c00081e)
#define MPI_DOUBLE_COMPLEX ((MPI_Datatype)0x4c001022)
#define MPI_INTEGER ((MPI_Datatype)0x4c00041b)

#define MPI_MAX ((MPI_Op)0x58000001)
#define MPI_MIN ((MPI_Op)0x58000002)
#define MPI_SUM ((MPI_Op)0x58000003)

#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3

#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *newcomm);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int *result);
MPI_Comm MPI_Comm_f2c(int fcomm);
int MPI_Comm_c2f(MPI_Comm comm);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int dims[], const int periods[], int reorder,
                    MPI_Comm *cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm *newcomm);
int MPI_Dims_create(int nnodes, int ndims, int dims[]);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root,
               MPI_Comm comm);
int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Alltoallv(const void *send, const int scounts[], const int sdispls[], MPI_Datatype stype,
                  void *recv, const int rcounts[], const int rdispls[], MPI_Datatype rtype,
                  MPI_Comm comm);
double MPI_Wtime(void);

#ifdef __cplusplus
}
#endif
#endif
