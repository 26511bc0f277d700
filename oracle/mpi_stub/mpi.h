/* Compile-only MPI stand-in used to build the reference library for the
 * single-process oracle.  The single-node `Graph::pattern_matching` path
 * never calls MPI; `Graphmpi::get_loop` is a no-op unless `set_loop_flag`
 * ran (reference src/graphmpi.cpp:207-213).  Every function here is a no-op
 * that reports a one-rank world, so the distributed path, if it were ever
 * entered, would behave as a single rank. */
#pragma once

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_UNSIGNED 0
#define MPI_ANY_SOURCE (-1)
#define MPI_THREAD_FUNNELED 1
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

static inline int MPI_Init_thread(int*, char***, int, int* provided) { if (provided) *provided = MPI_THREAD_FUNNELED; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Test(MPI_Request*, int* flag, MPI_Status*) { *flag = 0; return 0; }
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
