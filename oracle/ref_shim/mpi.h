/*
 * Single-process MPI stand-in used only to compile the unmodified CAPS
 * sources on one rank (oracle/build_ref.sh).  Test infrastructure: it is
 * never linked into the product library.
 *
 * One rank: size 1, rank 0; barriers, broadcasts and communicator set-up
 * are no-ops.  Point-to-point and collective data movement is never reached
 * on one rank by the 'd' path; if it is, the process aborts.
 */
#ifndef CAPS_ORACLE_MPI_STUB_H
#define CAPS_ORACLE_MPI_STUB_H
/* standard headers first: the CAPS library.h defines a max() macro */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <limits>
#include <algorithm>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

static inline void caps_mpi_stub_abort(const char *what) {
  fprintf(stderr, "single-rank MPI stand-in: %s needs more than one rank\n", what);
  abort();
}
static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Comm_group(MPI_Comm, MPI_Group *g) { *g = 0; return 0; }
static inline int MPI_Group_incl(MPI_Group, int, const int *, MPI_Group *g) { *g = 0; return 0; }
static inline int MPI_Comm_create(MPI_Comm, MPI_Group, MPI_Comm *c) { *c = 0; return 0; }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { caps_mpi_stub_abort("MPI_Send"); return 1; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { caps_mpi_stub_abort("MPI_Recv"); return 1; }
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { caps_mpi_stub_abort("MPI_Isend"); return 1; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { caps_mpi_stub_abort("MPI_Irecv"); return 1; }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { caps_mpi_stub_abort("MPI_Wait"); return 1; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { caps_mpi_stub_abort("MPI_Waitall"); return 1; }
static inline int MPI_Alltoall(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm) { caps_mpi_stub_abort("MPI_Alltoall"); return 1; }
static inline int MPI_Scatter(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm) { caps_mpi_stub_abort("MPI_Scatter"); return 1; }
static inline int MPI_Gather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm) { caps_mpi_stub_abort("MPI_Gather"); return 1; }
#endif
