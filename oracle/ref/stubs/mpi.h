/*
  Single-rank MPI stand-in used only to compile the reference TACS sources
  into a CPU checker library (oracle/_ref).  Test infrastructure: nothing in
  the shipped package includes this header.

  Semantics: one process, rank 0 of size 1.  Collectives copy the send buffer
  into the receive buffer; point-to-point messages can only be sent to self
  and are matched through a small in-process queue (ref_stubs.cpp).  Parallel
  file I/O aborts.
*/
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_File;
typedef long long MPI_Offset;
typedef long long MPI_Aint;

typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_bytes;
} MPI_Status;

typedef void MPI_User_function(void *, void *, int *, MPI_Datatype *);

#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_SELF ((MPI_Comm)2)
#define MPI_COMM_NULL ((MPI_Comm)0)

/* Datatype handles encode their byte size in the low 8 bits */
#define MPI_CHAR ((MPI_Datatype)(0x100 | 1))
#define MPI_BYTE ((MPI_Datatype)(0x200 | 1))
#define MPI_INT ((MPI_Datatype)(0x300 | 4))
#define MPI_FLOAT ((MPI_Datatype)(0x400 | 4))
#define MPI_DOUBLE ((MPI_Datatype)(0x500 | 8))
#define MPI_DOUBLE_COMPLEX ((MPI_Datatype)(0x600 | 16))
#define MPI_LONG ((MPI_Datatype)(0x700 | 8))
#define MPI_UNSIGNED ((MPI_Datatype)(0x800 | 4))

#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_PROD ((MPI_Op)4)
#define MPI_LOR ((MPI_Op)5)
#define MPI_LAND ((MPI_Op)6)

#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_REQUEST_NULL ((MPI_Request)(-1))
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_SUCCESS 0
#define MPI_UNDEFINED (-32766)
#define MPI_MAX_ERROR_STRING 256
#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1

int MPI_Init(int *argc, char ***argv);
int MPI_Initialized(int *flag);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int *result);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *out);
int MPI_Comm_free(MPI_Comm *comm);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);
int MPI_Error_string(int code, char *str, int *len);
int MPI_Op_create(MPI_User_function *fn, int commute, MPI_Op *op);
int MPI_Op_free(MPI_Op *op);

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root,
              MPI_Comm comm);
int MPI_Alltoall(const void *sendbuf, int scount, MPI_Datatype stype,
                 void *recvbuf, int rcount, MPI_Datatype rtype, MPI_Comm comm);
int MPI_Alltoallv(const void *sendbuf, const int *scounts, const int *sdispls,
                  MPI_Datatype stype, void *recvbuf, const int *rcounts,
                  const int *rdispls, MPI_Datatype rtype, MPI_Comm comm);
int MPI_Allgather(const void *sendbuf, int scount, MPI_Datatype stype,
                  void *recvbuf, int rcount, MPI_Datatype rtype,
                  MPI_Comm comm);
int MPI_Gather(const void *sendbuf, int scount, MPI_Datatype stype,
               void *recvbuf, int rcount, MPI_Datatype rtype, int root,
               MPI_Comm comm);
int MPI_Gatherv(const void *sendbuf, int scount, MPI_Datatype stype,
                void *recvbuf, const int *rcounts, const int *displs,
                MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Scatter(const void *sendbuf, int scount, MPI_Datatype stype,
                void *recvbuf, int rcount, MPI_Datatype rtype, int root,
                MPI_Comm comm);
int MPI_Scatterv(const void *sendbuf, const int *scounts, const int *displs,
                 MPI_Datatype stype, void *recvbuf, int rcount,
                 MPI_Datatype rtype, int root, MPI_Comm comm);

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag,
             MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag,
             MPI_Comm comm, MPI_Status *status);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest,
              int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status *status);
int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *statuses);
int MPI_Waitany(int n, MPI_Request *reqs, int *index, MPI_Status *status);

int MPI_File_open(MPI_Comm comm, const char *name, int amode, MPI_Info info,
                  MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype,
                      MPI_Datatype filetype, const char *datarep,
                      MPI_Info info);
int MPI_File_set_size(MPI_File fh, MPI_Offset size);
int MPI_File_write(MPI_File fh, const void *buf, int count, MPI_Datatype type,
                   MPI_Status *status);
int MPI_File_read(MPI_File fh, void *buf, int count, MPI_Datatype type,
                  MPI_Status *status);
int MPI_File_write_at_all(MPI_File fh, MPI_Offset off, const void *buf,
                          int count, MPI_Datatype type, MPI_Status *status);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int count,
                         MPI_Datatype type, MPI_Status *status);

#ifdef __cplusplus
}
#endif

#endif /* ORACLE_STUB_MPI_H */
