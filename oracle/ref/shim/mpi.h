/* Single-rank stand-in for the MPI calls made by the reference (counted by
 * grep over SourceFiles/: Init, Finalize, Comm_rank/size, Bcast, Reduce,
 * Allreduce, Send, Recv, Wtime, Comm_c2f).  With one rank every collective is
 * a copy or a no-op; Send/Recv are unreachable at one rank.
 * Test infrastructure for building the reference as the oracle, not product code. */
#pragma once
#include <string.h>
#include <time.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int dummy; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 10
#define MPI_MAX 11
#define MPI_MIN 12
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
static inline size_t pdx_mpi_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(double); }
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != r && n > 0) memmove(r, s, (size_t)n * pdx_mpi_size(t)); return 0; }
static inline int MPI_Allreduce(const void* s, void* r, long long n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != r && n > 0) memmove(r, s, (size_t)n * pdx_mpi_size(t)); return 0; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline double MPI_Wtime() { struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts); return ts.tv_sec + 1e-9 * ts.tv_nsec; }
static inline int MPI_Comm_c2f(MPI_Comm c) { return c; }
