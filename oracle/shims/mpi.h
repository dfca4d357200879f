/* Single-rank MPI shim: collectives are identities on one rank. */
#ifndef MXS_MPI_H
#define MXS_MPI_H
#include <stddef.h>
typedef int MPI_Comm;
typedef int MPI_Datatype; /* low byte = element size in bytes */
typedef int MPI_Op;
typedef int MPI_Info;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_BYTE ((MPI_Datatype)0x101)
#define MPI_CHAR ((MPI_Datatype)0x201)
#define MPI_C_BOOL ((MPI_Datatype)0x301)
#define MPI_INT ((MPI_Datatype)0x404)
#define MPI_FLOAT ((MPI_Datatype)0x504)
#define MPI_UNSIGNED ((MPI_Datatype)0x604)
#define MPI_LONG ((MPI_Datatype)0x708)
#define MPI_DOUBLE ((MPI_Datatype)0x808)
#define MPI_LONG_LONG ((MPI_Datatype)0x908)
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)0xa08)
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_LAND ((MPI_Op)4)
#define MPI_LOR ((MPI_Op)5)
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype dt, int root, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int scount, MPI_Datatype sdt, void* recvbuf, int rcount, MPI_Datatype rdt,
                  MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype dt, int src, int tag, MPI_Comm comm, MPI_Status* st);
int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype sdt, int dest, int stag, void* rbuf, int rcount,
                 MPI_Datatype rdt, int src, int rtag, MPI_Comm comm, MPI_Status* st);
int MPI_Barrier(MPI_Comm comm);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
#endif
