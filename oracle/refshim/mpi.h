/*
 * mpi.h -- MPI header for building the reference library here (oracle/_ref).
 * TEST INFRASTRUCTURE ONLY.
 *
 * The single-rank shim of include/mpi.h (rank 0 of 1; collectives copy send to receive), plus
 * the point-to-point routines that the reference's unused MPI_Alltoallv4 helper names
 * (build/exec.C:2343-2356).  On one rank a message can only go to itself: mpi_p2p.c matches a
 * send with the receive posted before it.
 */
#ifndef ORC_REF_MPI_H
#define ORC_REF_MPI_H
#include "../../include/mpi.h"
#ifdef __cplusplus
extern "C" {
#endif
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-2)
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]);
int MPI_Cart_rank(MPI_Comm comm, const int coords[], int *rank);
#ifdef __cplusplus
}
#endif
#endif
