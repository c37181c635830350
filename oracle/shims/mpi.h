/*
 * mpi.h -- single-rank loopback stand-in for the MPI calls cpic makes, so
 * that the reference's own sources build and run in one process.
 * TEST INFRASTRUCTURE ONLY (oracle/_ref).
 *
 * Rank 0 of 1.  Point-to-point sends are copied into a FIFO keyed by tag
 * and received by tag (the periodic self-exchange cpic performs on one
 * rank, src/comm_field.c:20-201); collectives and waits do nothing.
 */
#ifndef ORC_SHIM_MPI_H
#define ORC_SHIM_MPI_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef void *MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *) 0)
#define MPI_REQUEST_NULL ((MPI_Request) 0)
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
#define MPI_DOUBLE 1
#define MPI_BYTE 2
#define MPI_INT 3
#define MPI_LONG 4

int MPI_Init(int *argc, char ***argv);
int MPI_Init_thread(int *argc, char ***argv, int required, int *provided);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
		MPI_Request *req);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
		MPI_Status *status);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);

#endif
