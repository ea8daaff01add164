/*
 * mpi.h -- a single-process MPI stand-in used only to compile and run the
 * reference's own CPU oracle (gpu/Mugs.cc) as the checker for this
 * project's oracle.  Each MPI rank is a thread of one process; point-to-point
 * messages are copied eagerly into the destination's queue and matched in
 * post order per (source, tag), which gives MPI's non-overtaking order.
 *
 * Covers exactly what gpu/Mugs.cc calls: MPI_Comm_rank, MPI_Comm_size,
 * MPI_Irecv, MPI_Isend, MPI_Waitall.
 */
#pragma once
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct mpistub_request *MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUCCESS 0
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]);

/* run fn(rank, arg) on `size` threads, one per rank; returns when all end */
void mpistub_run(int size, void (*fn)(int rank, void *arg), void *arg);

#ifdef __cplusplus
}
#endif
