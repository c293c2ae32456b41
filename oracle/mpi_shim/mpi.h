/*
 * Single-rank stand-in for the handful of MPI calls the MDACP sources make.
 *
 * Test infrastructure only: it lets the reference sources build and run as
 * `mpirun -np 1` would, without an MPI installation.  With one rank every
 * point-to-point exchange is a copy to self and every reduction is the
 * identity, which is exactly what MPI does at one rank.  Counts are taken from
 * the SEND side (communicator.h:15-19 sends MPI_BYTE but receives with the
 * byte count typed as MPI_DOUBLE; at one rank only the send size is real).
 */
#ifndef MDG_ORACLE_MPI_SHIM_H
#define MDG_ORACLE_MPI_SHIM_H

#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_BYTE 1
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_UNSIGNED_LONG 9
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_LOR 2

static inline size_t mdg_shim_size(MPI_Datatype t) {
  return t == MPI_UNSIGNED_LONG ? sizeof(unsigned long) : (size_t)t;
}
static inline void mdg_shim_copy(void *dst, const void *src, int n, MPI_Datatype t) {
  if (n > 0 && dst != src) memcpy(dst, src, (size_t)n * mdg_shim_size(t));
}
static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Sendrecv(const void *sb, int sc, MPI_Datatype st, int, int, void *rb, int, MPI_Datatype,
                               int, int, MPI_Comm, MPI_Status *) {
  mdg_shim_copy(rb, sb, sc, st);
  return 0;
}
static inline int MPI_Allreduce(const void *sb, void *rb, int c, MPI_Datatype t, MPI_Op, MPI_Comm) {
  mdg_shim_copy(rb, sb, c, t);
  return 0;
}
static inline int MPI_Allgather(const void *sb, int sc, MPI_Datatype st, void *rb, int, MPI_Datatype, MPI_Comm) {
  mdg_shim_copy(rb, sb, sc, st);
  return 0;
}
static inline int MPI_Gather(const void *sb, int sc, MPI_Datatype st, void *rb, int, MPI_Datatype, int, MPI_Comm) {
  mdg_shim_copy(rb, sb, sc, st);
  return 0;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }

/* Balanced factorisation in non-increasing order, as MPI_Dims_create returns
 * for an all-zero dims array. */
static inline int MPI_Dims_create(int nnodes, int ndims, int *dims) {
  for (int d = 0; d < ndims; d++) dims[d] = 1;
  int f[64], nf = 0, n = nnodes;
  for (int p = 2; p * p <= n; p++)
    while (n % p == 0) { f[nf++] = p; n /= p; }
  if (n > 1) f[nf++] = n;
  for (int k = nf - 1; k >= 0; k--) { /* largest factor to the smallest dim */
    int m = 0;
    for (int d = 1; d < ndims; d++) if (dims[d] < dims[m]) m = d;
    dims[m] *= f[k];
  }
  for (int a = 0; a < ndims; a++)
    for (int b = a + 1; b < ndims; b++)
      if (dims[b] > dims[a]) { int t = dims[a]; dims[a] = dims[b]; dims[b] = t; }
  return 0;
}

#endif
