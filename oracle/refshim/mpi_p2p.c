/*
 * Point-to-point MPI routines on one rank for the reference build (oracle/_ref).
 * TEST INFRASTRUCTURE ONLY.  A receive is posted into a small table; a send to rank 0 fills
 * the oldest posted receive whose tag matches; Waitall has nothing left to wait for.
 */
#include "mpi.h"

#include <stdio.h>
#include <string.h>

#define ORC_MAX_PENDING 64
static struct {
  void *buf;
  int bytes, tag, used;
} pend[ORC_MAX_PENDING];

static int tsize(MPI_Datatype t) { return (int)(t & 0xff00) >> 8; }

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request *req)
{
  int i;
  (void)source; (void)comm;
  for (i = 0; i < ORC_MAX_PENDING; i++)
    if (!pend[i].used) {
      pend[i].buf = buf;
      pend[i].bytes = count * tsize(type);
      pend[i].tag = tag;
      pend[i].used = 1;
      *req = i;
      return MPI_SUCCESS;
    }
  fprintf(stderr, "MPI_Irecv: too many pending receives on a single rank\n");
  return 1;
}

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm)
{
  int i, bytes = count * tsize(type);
  (void)comm;
  if (dest != 0) return 1;
  for (i = 0; i < ORC_MAX_PENDING; i++)
    if (pend[i].used && (pend[i].tag == MPI_ANY_TAG || pend[i].tag == tag)) {
      memcpy(pend[i].buf, buf, (size_t)(bytes < pend[i].bytes ? bytes : pend[i].bytes));
      pend[i].used = 0;
      return MPI_SUCCESS;
    }
  fprintf(stderr, "MPI_Send: no matching receive posted on a single rank\n");
  return 1;
}

int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[])
{
  (void)count; (void)reqs; (void)statuses;
  return MPI_SUCCESS;
}

int MPI_Cart_rank(MPI_Comm comm, const int coords[], int *rank)
{
  (void)comm; (void)coords;
  *rank = 0;
  return MPI_SUCCESS;
}
