/* Single-rank stand-in for the MPI calls the reference's nb_main.cpp names (TEST
 * INFRASTRUCTURE ONLY).  The oracle driver never calls NomadBody::run, so none of
 * these runs during a check; they exist so that the unmodified file compiles.  With
 * one rank an all-reduce is a copy and a barrier returns at once. */
#ifndef NOMAD_REFSHIM_MPI_H_
#define NOMAD_REFSHIM_MPI_H_

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_LONG_LONG 9
#define MPI_CHAR 1
#define MPI_SUM 0
#define MPI_THREAD_MULTIPLE 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_MAX_PROCESSOR_NAME 256

static inline int refshim_mpi_size(MPI_Datatype t) { return t == MPI_LONG_LONG ? 8 : t; }
static inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  memmove(out, in, (size_t)count * (size_t)refshim_mpi_size(t));
  return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }

#endif
