/* Minimal single-process MPI stand-ins so that the reference's host-side C
 * files compile for the oracle check (one rank, no communication). */
#ifndef RO_STUB_MPI_H
#define RO_STUB_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_MAX 2
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
void ro_stub_abort(int code);
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; ro_stub_abort(code); return 0; }
static inline double MPI_Wtime(void) { return 0.0; }
/* one rank: the reduction is a copy (doubles or ints) */
static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype dt,
                                MPI_Op op, MPI_Comm c) {
  int k;
  (void)op; (void)c;
  if (dt == MPI_DOUBLE)
    for (k = 0; k < count; k++) ((double *)out)[k] = ((const double *)in)[k];
  else
    for (k = 0; k < count; k++) ((int *)out)[k] = ((const int *)in)[k];
  return 0;
}
#endif
