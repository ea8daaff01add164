// mpi_single.cc -- the one-rank MPI stand-in of mpi.h.
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>

namespace {

void only_null(const char *what, int peer)
{
  if (peer == MPI_PROC_NULL) return;
  std::fprintf(stderr, "mpi_single: %s with peer %d: only MPI_PROC_NULL exists in a one-rank world\n", what, peer);
  std::abort();
}

int type_bytes(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }

}  // namespace

extern "C" {

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_split_type(MPI_Comm, int, int, MPI_Info, MPI_Comm *out) { *out = MPI_COMM_WORLD; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op, int, MPI_Comm)
{
  std::memmove(recv, send, (size_t)count * type_bytes(type));
  return MPI_SUCCESS;
}

double MPI_Wtime(void)
{
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Irecv(void *, int, MPI_Datatype, int source, int, MPI_Comm, MPI_Request *req)
{
  only_null("MPI_Irecv", source);
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

int MPI_Isend(const void *, int, MPI_Datatype, int dest, int, MPI_Comm, MPI_Request *req)
{
  only_null("MPI_Isend", dest);
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

int MPI_Waitall(int, MPI_Request[], MPI_Status[]) { return MPI_SUCCESS; }

}  // extern "C"
