/*
 * mpi.h -- a one-rank MPI stand-in, used only to build and run the
 * reference's own CUDA executables (gpu/main.cc with a gpu/v-* strategy) on
 * a single GPU as a baseline.  The process is rank 0 of a world of size 1.
 * On a 1x1x1 task grid every neighbour of the reference's Faces and Mugs is
 * MPI_PROC_NULL (gpu/v-26-messages/Faces.cc:92-103, gpu/Mugs.cc:72-83), so
 * point-to-point calls only ever name MPI_PROC_NULL: they complete at once
 * and leave the receive buffer untouched, as MPI specifies.  Any other peer
 * aborts with a message.  Collectives over one rank copy or do nothing.
 *
 * Covers what those files call: MPI_Init, MPI_Finalize, MPI_Comm_size,
 * MPI_Comm_rank, MPI_Comm_split_type, MPI_Barrier, MPI_Bcast, MPI_Reduce,
 * MPI_Wtime, MPI_Irecv, MPI_Isend, MPI_Waitall.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_REQUEST_NULL 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_SUCCESS 0
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_split_type(MPI_Comm comm, int type, int key, MPI_Info info, MPI_Comm *out);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]);

#ifdef __cplusplus
}
#endif
