/* Single-rank stand-in for the MPI interface the reference's hot-path TUs
 * use (TEST INFRASTRUCTURE: lets oracle/ref.mk compile the reference's own
 * step functions in place for parity pinning; never part of the product).
 *
 * With one rank every collective is a copy of the caller's own contribution
 * (or nothing at all with MPI_IN_PLACE), which is what an MPI library returns
 * for a one-process communicator.  Point-to-point calls have no partner and
 * abort.  A datatype is its size in bytes. */
#ifndef CMCREF_SHIM_MPI_H
#define CMCREF_SHIM_MPI_H
#include <stddef.h>

typedef int MPI_Comm;
typedef long MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Group;
typedef int MPI_File;
typedef int MPI_Request;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_DATATYPE_NULL ((MPI_Datatype)0)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_IN_PLACE ((void *)-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Abort(MPI_Comm comm, int code);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Exscan(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Gather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm comm);
int MPI_Allgatherv(const void *s, int sc, MPI_Datatype st, void *r, const int *rcs, const int *displs,
                   MPI_Datatype rt, MPI_Comm comm);
int MPI_Alltoall(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm comm);
int MPI_Alltoallv(const void *s, const int *scs, const int *sdispls, MPI_Datatype st, void *r, const int *rcs,
                  const int *rdispls, MPI_Datatype rt, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st);
int MPI_Sendrecv(const void *s, int sc, MPI_Datatype st, int dest, int stag, void *r, int rc, MPI_Datatype rt,
                 int src, int rtag, MPI_Comm comm, MPI_Status *status);
int MPI_Comm_group(MPI_Comm comm, MPI_Group *g);
int MPI_Group_incl(MPI_Group g, int n, const int ranks[], MPI_Group *out);
int MPI_Comm_create(MPI_Comm comm, MPI_Group g, MPI_Comm *out);
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *t);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);
int MPI_Type_size(MPI_Datatype t, int *size);
#endif
