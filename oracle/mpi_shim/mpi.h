/*
 * Serial stand-in for the handful of MPI calls UNAP's x86 sources make.
 *
 * Test infrastructure only: it lets the reference library be compiled as a
 * single-rank CPU oracle (oracle/_ref) without an MPI installation.  With one
 * rank every collective is a copy and every point-to-point call is a no-op,
 * which is exactly the PARRUN == false path of the reference
 * (src/base/mpi/unapMPI.cpp:9-57 sets parRun_ only when nProcs_ > 1).
 */
#ifndef UNAP_ORACLE_MPI_SHIM_H
#define UNAP_ORACLE_MPI_SHIM_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0

#define MPI_INT 1
#define MPI_LONG 2
#define MPI_DOUBLE 3
#define MPI_FLOAT 4
#define MPI_CXX_BOOL 5
#define MPI_CHAR 6

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_LOR 3

#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

static inline size_t unap_shim_type_size(MPI_Datatype t)
{
    switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_LONG: return sizeof(long);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_FLOAT: return sizeof(float);
    case MPI_CXX_BOOL: return sizeof(bool);
    default: return 1;
    }
}

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Initialized(int* flag) { *flag = 1; return MPI_SUCCESS; }
static inline int MPI_Finalized(int* flag) { *flag = 0; return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count,
                                MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t)count * unap_shim_type_size(t));
    return MPI_SUCCESS;
}

static inline int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype st,
                                void* recvbuf, int, MPI_Datatype, MPI_Comm)
{
    if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t)sendcount * unap_shim_type_size(st));
    return MPI_SUCCESS;
}

static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r)
{ *r = 0; return MPI_SUCCESS; }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r)
{ *r = 0; return MPI_SUCCESS; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return MPI_SUCCESS; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }

#endif
