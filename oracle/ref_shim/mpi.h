// Single-rank stand-in for <mpi.h> (test infrastructure only).  With one
// rank every reference collective reduces to a copy, which is exactly the
// reference's own behaviour at MPI_Comm_size == 1.
#ifndef A2C_REF_SHIM_MPI_H
#define A2C_REF_SHIM_MPI_H
#include <cstdlib>
#include <cstring>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 1
#define MPI_MAX 2
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != r) std::memcpy(r, s, (size_t)n * (size_t)t);
  return 0;
}
#endif
