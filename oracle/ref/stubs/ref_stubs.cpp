/*
  Link-time stand-ins for the reference TACS build used as a CPU checker
  (oracle/_ref).  Test infrastructure only.

  - Single-rank MPI: rank 0 of 1; collectives copy; self-addressed
    point-to-point messages go through an in-process queue.
  - The six BLAS level-1/2 routines the reference's vector and assembly code
    call (dot, nrm2, axpy, scal, copy, gemv), written from their reference
    definitions, in a real and a complex flavour selected by TACS_USE_COMPLEX.
  - LAPACK and METIS entry points that are off the checked path abort.
*/
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <vector>

extern "C" {
#include "metis.h"
}
#include "mpi.h"

#ifdef TACS_USE_COMPLEX
typedef std::complex<double> Scalar;
#else
typedef double Scalar;
#endif

static void stub_abort(const char *name) {
  fprintf(stderr, "oracle stub: %s is not available in the checker build\n",
          name);
  abort();
}

static size_t type_size(MPI_Datatype t) { return (size_t)(t & 0xff); }

/* ---------------------------- MPI ----------------------------------- */
namespace {
struct Message {
  int tag;
  std::vector<char> data;
};
struct PendingRecv {
  void *buf;
  size_t max_bytes;
  int tag;
  bool done;
};
std::deque<Message> g_queue;
std::vector<PendingRecv> g_recvs;

bool try_match(PendingRecv &r) {
  for (auto it = g_queue.begin(); it != g_queue.end(); ++it) {
    if (r.tag == MPI_ANY_TAG || it->tag == r.tag) {
      size_t n = it->data.size() < r.max_bytes ? it->data.size() : r.max_bytes;
      if (n) memcpy(r.buf, it->data.data(), n);
      g_queue.erase(it);
      r.done = true;
      return true;
    }
  }
  return false;
}
}  // namespace

extern "C" {

int MPI_Init(int *, char ***) { return 0; }
int MPI_Initialized(int *flag) {
  *flag = 1;
  return 0;
}
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm, int code) {
  fprintf(stderr, "MPI_Abort(%d)\n", code);
  abort();
}
int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = 0;
  return 0;
}
int MPI_Comm_size(MPI_Comm, int *size) {
  *size = 1;
  return 0;
}
int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int *result) {
  *result = (a == b) ? MPI_IDENT : MPI_CONGRUENT;
  return 0;
}
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *out) {
  *out = comm;
  return 0;
}
int MPI_Comm_free(MPI_Comm *comm) {
  *comm = MPI_COMM_NULL;
  return 0;
}
double MPI_Wtime(void) {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Error_string(int code, char *str, int *len) {
  *len = snprintf(str, MPI_MAX_ERROR_STRING, "stub MPI error %d", code);
  return 0;
}
int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) {
  static int next = 100;
  *op = next++;
  return 0;
}
int MPI_Op_free(MPI_Op *op) {
  *op = 0;
  return 0;
}

static void copy_buf(const void *src, void *dst, size_t bytes) {
  if (src == MPI_IN_PLACE || src == dst || bytes == 0) return;
  memmove(dst, src, bytes);
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype type, MPI_Op, MPI_Comm) {
  copy_buf(sendbuf, recvbuf, (size_t)count * type_size(type));
  return 0;
}
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype type, MPI_Op, int, MPI_Comm) {
  copy_buf(sendbuf, recvbuf, (size_t)count * type_size(type));
  return 0;
}
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Alltoall(const void *sendbuf, int scount, MPI_Datatype stype,
                 void *recvbuf, int, MPI_Datatype, MPI_Comm) {
  copy_buf(sendbuf, recvbuf, (size_t)scount * type_size(stype));
  return 0;
}
int MPI_Alltoallv(const void *sendbuf, const int *scounts, const int *sdispls,
                  MPI_Datatype stype, void *recvbuf, const int *,
                  const int *rdispls, MPI_Datatype rtype, MPI_Comm) {
  size_t ss = type_size(stype), rs = type_size(rtype);
  copy_buf((const char *)sendbuf + (size_t)sdispls[0] * ss,
           (char *)recvbuf + (size_t)rdispls[0] * rs, (size_t)scounts[0] * ss);
  return 0;
}
int MPI_Allgather(const void *sendbuf, int scount, MPI_Datatype stype,
                  void *recvbuf, int, MPI_Datatype, MPI_Comm) {
  copy_buf(sendbuf, recvbuf, (size_t)scount * type_size(stype));
  return 0;
}
int MPI_Gather(const void *sendbuf, int scount, MPI_Datatype stype,
               void *recvbuf, int, MPI_Datatype, int, MPI_Comm) {
  copy_buf(sendbuf, recvbuf, (size_t)scount * type_size(stype));
  return 0;
}
int MPI_Gatherv(const void *sendbuf, int scount, MPI_Datatype stype,
                void *recvbuf, const int *, const int *displs,
                MPI_Datatype rtype, int, MPI_Comm) {
  copy_buf(sendbuf, (char *)recvbuf + (size_t)displs[0] * type_size(rtype),
           (size_t)scount * type_size(stype));
  return 0;
}
int MPI_Scatter(const void *sendbuf, int, MPI_Datatype, void *recvbuf,
                int rcount, MPI_Datatype rtype, int, MPI_Comm) {
  copy_buf(sendbuf, recvbuf, (size_t)rcount * type_size(rtype));
  return 0;
}
int MPI_Scatterv(const void *sendbuf, const int *, const int *displs,
                 MPI_Datatype stype, void *recvbuf, int rcount,
                 MPI_Datatype rtype, int, MPI_Comm) {
  copy_buf((const char *)sendbuf + (size_t)displs[0] * type_size(stype),
           recvbuf, (size_t)rcount * type_size(rtype));
  return 0;
}

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag,
             MPI_Comm) {
  if (dest != 0) stub_abort("MPI_Send to a rank other than 0");
  Message m;
  m.tag = tag;
  m.data.assign((const char *)buf,
                (const char *)buf + (size_t)count * type_size(type));
  g_queue.push_back(std::move(m));
  return 0;
}
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest,
              int tag, MPI_Comm comm, MPI_Request *req) {
  MPI_Send(buf, count, type, dest, tag, comm);
  *req = MPI_REQUEST_NULL;
  return 0;
}
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag,
              MPI_Comm, MPI_Request *req) {
  if (source != 0 && source != MPI_ANY_SOURCE)
    stub_abort("MPI_Irecv from a rank other than 0");
  PendingRecv r = {buf, (size_t)count * type_size(type), tag, false};
  try_match(r);
  g_recvs.push_back(r);
  *req = (MPI_Request)(g_recvs.size() - 1);
  return 0;
}
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag,
             MPI_Comm comm, MPI_Status *status) {
  MPI_Request req;
  MPI_Irecv(buf, count, type, source, tag, comm, &req);
  return MPI_Wait(&req, status);
}
int MPI_Probe(int, int tag, MPI_Comm, MPI_Status *status) {
  for (auto &m : g_queue) {
    if (tag == MPI_ANY_TAG || m.tag == tag) {
      if (status) {
        status->MPI_SOURCE = 0;
        status->MPI_TAG = m.tag;
        status->MPI_ERROR = 0;
        status->count_bytes = (int)m.data.size();
      }
      return 0;
    }
  }
  stub_abort("MPI_Probe with no matching self message");
  return 1;
}
int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count) {
  *count = status->count_bytes / (int)type_size(type);
  return 0;
}
int MPI_Wait(MPI_Request *req, MPI_Status *status) {
  if (*req != MPI_REQUEST_NULL) {
    PendingRecv &r = g_recvs[*req];
    if (!r.done && !try_match(r)) stub_abort("MPI_Wait on an unmatched receive");
    *req = MPI_REQUEST_NULL;
  }
  if (status) {
    status->MPI_SOURCE = 0;
    status->MPI_ERROR = 0;
  }
  return 0;
}
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *statuses) {
  for (int i = 0; i < n; i++) MPI_Wait(&reqs[i], statuses ? &statuses[i] : 0);
  bool any_open = false;
  for (auto &r : g_recvs) any_open |= !r.done;
  if (!any_open) g_recvs.clear();
  return 0;
}
int MPI_Waitany(int n, MPI_Request *reqs, int *index, MPI_Status *status) {
  for (int i = 0; i < n; i++) {
    if (reqs[i] != MPI_REQUEST_NULL) {
      *index = i;
      return MPI_Wait(&reqs[i], status);
    }
  }
  *index = MPI_UNDEFINED;
  return 0;
}

int MPI_File_open(MPI_Comm, const char *, int, MPI_Info, MPI_File *) {
  stub_abort("MPI_File_open");
  return 1;
}
int MPI_File_close(MPI_File *) { return 0; }
int MPI_File_set_view(MPI_File, MPI_Offset, MPI_Datatype, MPI_Datatype,
                      const char *, MPI_Info) {
  stub_abort("MPI_File_set_view");
  return 1;
}
int MPI_File_set_size(MPI_File, MPI_Offset) {
  stub_abort("MPI_File_set_size");
  return 1;
}
int MPI_File_write(MPI_File, const void *, int, MPI_Datatype, MPI_Status *) {
  stub_abort("MPI_File_write");
  return 1;
}
int MPI_File_read(MPI_File, void *, int, MPI_Datatype, MPI_Status *) {
  stub_abort("MPI_File_read");
  return 1;
}
int MPI_File_write_at_all(MPI_File, MPI_Offset, const void *, int,
                          MPI_Datatype, MPI_Status *) {
  stub_abort("MPI_File_write_at_all");
  return 1;
}
int MPI_File_read_at_all(MPI_File, MPI_Offset, void *, int, MPI_Datatype,
                         MPI_Status *) {
  stub_abort("MPI_File_read_at_all");
  return 1;
}

/* ---------------------------- METIS --------------------------------- */
int METIS_SetDefaultOptions(int *options) {
  for (int i = 0; i < METIS_NOPTIONS; i++) options[i] = -1;
  return 1;
}
int METIS_PartGraphRecursive(int *, int *, int *, int *, int *, int *, int *,
                             int *, double *, double *, int *, int *, int *) {
  stub_abort("METIS_PartGraphRecursive");
  return 0;
}
int METIS_PartGraphKway(int *, int *, int *, int *, int *, int *, int *,
                        int *, double *, double *, int *, int *, int *) {
  stub_abort("METIS_PartGraphKway");
  return 0;
}
int METIS_NodeND(int *, int *, int *, int *, int *, int *, int *) {
  stub_abort("METIS_NodeND");
  return 0;
}

/* ----------------------------- BLAS --------------------------------- */
#ifdef TACS_USE_COMPLEX
#define SDOT zdotu_
#define SNRM2 dznrm2_
#define SAXPY zaxpy_
#define SSCAL zscal_
#define SCOPY zcopy_
#define SGEMV zgemv_
#else
#define SDOT ddot_
#define SNRM2 dnrm2_
#define SAXPY daxpy_
#define SSCAL dscal_
#define SCOPY dcopy_
#define SGEMV dgemv_
#endif

Scalar SDOT(int *n, Scalar *x, int *incx, Scalar *y, int *incy) {
  Scalar s = 0.0;
  for (int i = 0; i < *n; i++) s += x[i * (*incx)] * y[i * (*incy)];
  return s;
}
double SNRM2(int *n, Scalar *x, int *incx) {
  /* Scaled sum of squares, as in the reference BLAS definition */
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < *n; i++) {
    Scalar v = x[i * (*incx)];
#ifdef TACS_USE_COMPLEX
    double parts[2] = {v.real(), v.imag()};
    for (int k = 0; k < 2; k++) {
      double a = parts[k];
#else
    {
      double a = v;
#endif
      if (a != 0.0) {
        double absa = a < 0 ? -a : a;
        if (scale < absa) {
          ssq = 1.0 + ssq * (scale / absa) * (scale / absa);
          scale = absa;
        } else {
          ssq += (absa / scale) * (absa / scale);
        }
      }
    }
  }
  return scale * __builtin_sqrt(ssq);
}
void SAXPY(int *n, Scalar *a, Scalar *x, int *incx, Scalar *y, int *incy) {
  for (int i = 0; i < *n; i++) y[i * (*incy)] += (*a) * x[i * (*incx)];
}
void SSCAL(int *n, Scalar *a, Scalar *x, int *incx) {
  for (int i = 0; i < *n; i++) x[i * (*incx)] *= (*a);
}
void SCOPY(int *n, Scalar *x, int *incx, Scalar *y, int *incy) {
  for (int i = 0; i < *n; i++) y[i * (*incy)] = x[i * (*incx)];
}
/* Column-major y = alpha*op(A)*x + beta*y */
void SGEMV(const char *trans, int *m, int *n, Scalar *alpha, Scalar *a,
           int *lda, Scalar *x, int *incx, Scalar *beta, Scalar *y,
           int *incy) {
  bool t = (trans[0] == 'T' || trans[0] == 't' || trans[0] == 'C' ||
            trans[0] == 'c');
  int leny = t ? *n : *m, lenx = t ? *m : *n;
  for (int i = 0; i < leny; i++) y[i * (*incy)] *= (*beta);
  if (!t) {
    for (int j = 0; j < lenx; j++) {
      Scalar tmp = (*alpha) * x[j * (*incx)];
      for (int i = 0; i < leny; i++) y[i * (*incy)] += tmp * a[i + j * (*lda)];
    }
  } else {
    for (int j = 0; j < leny; j++) {
      Scalar tmp = 0.0;
      for (int i = 0; i < lenx; i++) tmp += a[i + j * (*lda)] * x[i * (*incx)];
      y[j * (*incy)] += (*alpha) * tmp;
    }
  }
}

/* Off-path BLAS/LAPACK: abort if reached */
#define ABORT_STUB(name) \
  void name() { stub_abort(#name); }
#ifdef TACS_USE_COMPLEX
ABORT_STUB(zgemm_)
ABORT_STUB(ztrsm_)
ABORT_STUB(ztrsv_)
ABORT_STUB(ztbsv_)
ABORT_STUB(zsbmv_)
ABORT_STUB(zgbmv_)
ABORT_STUB(zgetrf_)
ABORT_STUB(zgetri_)
ABORT_STUB(zgetrs_)
ABORT_STUB(zgesv_)
ABORT_STUB(zpbtrf_)
ABORT_STUB(zstev_)
ABORT_STUB(zspsv_)
ABORT_STUB(zggev_)
#else
ABORT_STUB(dgemm_)
ABORT_STUB(dtrsm_)
ABORT_STUB(dtrsv_)
ABORT_STUB(dtbsv_)
ABORT_STUB(dsbmv_)
ABORT_STUB(dgbmv_)
ABORT_STUB(dgetrf_)
ABORT_STUB(dgetri_)
ABORT_STUB(dgetrs_)
ABORT_STUB(dgesv_)
ABORT_STUB(dpbtrf_)
ABORT_STUB(dstev_)
ABORT_STUB(dspsv_)
#endif
ABORT_STUB(dgeev_)
ABORT_STUB(dggev_)
ABORT_STUB(dstevr_)
ABORT_STUB(dsyev_)
ABORT_STUB(dsyevd_)
ABORT_STUB(dsygvd_)
ABORT_STUB(dspev_)
ABORT_STUB(dspgv_)
ABORT_STUB(dsbev_)
ABORT_STUB(dsbgv_)
ABORT_STUB(dsbgvx_)
ABORT_STUB(dpbsv_)
ABORT_STUB(dgelss_)

}  // extern "C"
