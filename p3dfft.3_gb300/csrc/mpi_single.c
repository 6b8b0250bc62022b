/*
 * Single-rank MPI shim (libp3dfft_mpi1.so), see include/mpi.h.  Every routine behaves as the
 * one-process case of the MPI standard: rank 0, size 1, reductions and all-to-alls copy the
 * send buffer to the receive buffer.
 */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static int dtype_size(MPI_Datatype t) { return (int)(t & 0xff00) >> 8; }

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm comm, int errorcode)
{
  (void)comm;
  fprintf(stderr, "MPI_Abort(%d) called on a single-rank run\n", errorcode);
  exit(errorcode ? errorcode : 1);
}
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *newcomm) { *newcomm = comm; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm *comm) { *comm = MPI_COMM_NULL; return MPI_SUCCESS; }
int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int *result)
{
  *result = (a == b) ? MPI_IDENT : MPI_CONGRUENT;
  return MPI_SUCCESS;
}
MPI_Comm MPI_Comm_f2c(int fcomm) { return (MPI_Comm)fcomm; }
int MPI_Comm_c2f(MPI_Comm comm) { return (int)comm; }
int MPI_Cart_create(MPI_Comm comm, int ndims, const int dims[], const int periods[], int reorder, MPI_Comm *cart)
{
  int i, n = 1;
  (void)periods; (void)reorder;
  for (i = 0; i < ndims; i++) n *= dims[i];
  if (n != 1) return 1;
  *cart = comm;
  return MPI_SUCCESS;
}
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[])
{
  int i;
  (void)comm; (void)rank;
  for (i = 0; i < maxdims; i++) coords[i] = 0;
  return MPI_SUCCESS;
}
int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm *newcomm)
{
  (void)remain_dims;
  *newcomm = comm;
  return MPI_SUCCESS;
}
int MPI_Dims_create(int nnodes, int ndims, int dims[])
{
  int i;
  (void)nnodes;
  for (i = 0; i < ndims; i++)
    if (dims[i] <= 0) dims[i] = 1;
  return MPI_SUCCESS;
}
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm)
{
  (void)buf; (void)count; (void)type; (void)root; (void)comm;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }
int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm)
{
  (void)op; (void)root; (void)comm;
  if (send != recv && recv) memmove(recv, send, (size_t)count * dtype_size(type));
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm)
{
  return MPI_Reduce(send, recv, count, type, op, 0, comm);
}
int MPI_Alltoallv(const void *send, const int scounts[], const int sdispls[], MPI_Datatype stype, void *recv,
                  const int rcounts[], const int rdispls[], MPI_Datatype rtype, MPI_Comm comm)
{
  (void)rcounts; (void)comm;
  memmove((char *)recv + (size_t)rdispls[0] * dtype_size(rtype), (const char *)send + (size_t)sdispls[0] * dtype_size(stype),
          (size_t)scounts[0] * dtype_size(stype));
  return MPI_SUCCESS;
}
double MPI_Wtime(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
