/* Single-rank MPI stand-in for compiling the reference solver as one process.
 *
 * Test infrastructure only: it lets the reference's own sources (which include
 * <mpi.h> unconditionally) build and run with one rank, so that the reference
 * itself can produce golden outputs.  Collectives on one rank reduce to a copy
 * of the send buffer into the receive buffer (nothing when MPI_IN_PLACE);
 * point-to-point calls have no peer and abort if ever reached. */
#ifndef PCFD_REFBUILD_MPI_H
#define PCFD_REFBUILD_MPI_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <complex>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
struct pcfd_mpi_double_int { double d; int i; };

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

enum {
  MPI_INT = 1, MPI_FLOAT, MPI_DOUBLE, MPI_DOUBLE_COMPLEX, MPI_COMPLEX, MPI_BYTE,
  MPI_DOUBLE_INT, MPI_CHAR, MPI_LONG, MPI_UNSIGNED
};
enum { MPI_SUM = 1, MPI_MAX, MPI_MIN, MPI_MINLOC, MPI_MAXLOC, MPI_PROD };

static inline size_t pcfd_mpi_type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_FLOAT: return sizeof(float);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_DOUBLE_COMPLEX: return sizeof(std::complex<double>);
    case MPI_COMPLEX: return sizeof(std::complex<float>);
    case MPI_BYTE: return 1;
    case MPI_CHAR: return 1;
    case MPI_DOUBLE_INT: return sizeof(pcfd_mpi_double_int);
    case MPI_LONG: return sizeof(long);
    case MPI_UNSIGNED: return sizeof(unsigned);
  }
  std::fprintf(stderr, "mpi stand-in: unknown datatype %d\n", t);
  std::abort();
}

static inline void pcfd_mpi_copy(const void* s, void* r, int count, MPI_Datatype t) {
  if (s == MPI_IN_PLACE || s == r || count <= 0) return;
  std::memmove(r, s, (size_t)count * pcfd_mpi_type_size(t));
}

static inline void pcfd_mpi_no_peer(const char* what) {
  std::fprintf(stderr, "mpi stand-in: %s has no peer in a single-rank run\n", what);
  std::abort();
}

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { std::exit(code ? code : 1); }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  pcfd_mpi_copy(s, r, n, t); return 0;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  pcfd_mpi_copy(s, r, n, t); return 0;
}
static inline int MPI_Allgather(const void* s, int ns, MPI_Datatype ts, void* r, int, MPI_Datatype, MPI_Comm) {
  pcfd_mpi_copy(s, r, ns, ts); return 0;
}
static inline int MPI_Alltoall(const void* s, int ns, MPI_Datatype ts, void* r, int, MPI_Datatype, MPI_Comm) {
  pcfd_mpi_copy(s, r, ns, ts); return 0;
}
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) {
  pcfd_mpi_no_peer("MPI_Isend"); return 1;
}
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) {
  pcfd_mpi_no_peer("MPI_Irecv"); return 1;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) {
  pcfd_mpi_no_peer("MPI_Send"); return 1;
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
  pcfd_mpi_no_peer("MPI_Recv"); return 1;
}
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
static inline double MPI_Wtime() { return 0.0; }

#endif
