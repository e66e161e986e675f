/* Single-rank MPI for the reference-as-oracle build (test infrastructure).
 * Collectives copy the send buffer to the receive buffer; point-to-point
 * traffic cannot happen with one rank and aborts if reached. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "include/mpi.h"

static size_t dt_size(MPI_Datatype t) { return (size_t)(t >> 4); }
static int copy_buf(const void *s, void *r, int n, MPI_Datatype t) {
  if (s == MPI_IN_PLACE || s == r || n <= 0) return MPI_SUCCESS;
  memcpy(r, s, (size_t)n * dt_size(t));
  return MPI_SUCCESS;
}
static int p2p(const char *who) {
  fprintf(stderr, "mpi_serial: %s reached with a single rank\n", who);
  abort();
  return -1;
}
int MPI_Init(int *a, char ***b) {
  (void)a;
  (void)b;
  return 0;
}
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm c, int e) {
  (void)c;
  fprintf(stderr, "mpi_serial: MPI_Abort(%d)\n", e);
  exit(e ? e : 1);
}
int MPI_Comm_rank(MPI_Comm c, int *r) {
  (void)c;
  *r = 0;
  return 0;
}
int MPI_Comm_size(MPI_Comm c, int *s) {
  (void)c;
  *s = 1;
  return 0;
}
int MPI_Barrier(MPI_Comm c) {
  (void)c;
  return 0;
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Error_string(int e, char *s, int *l) {
  *l = snprintf(s, MPI_MAX_ERROR_STRING, "mpi error %d", e);
  return 0;
}
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)o;
  (void)c;
  return copy_buf(s, r, n, t);
}
int MPI_Iallreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c,
                   MPI_Request *q) {
  *q = 0;
  return MPI_Allreduce(s, r, n, t, o, c);
}
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, int root, MPI_Comm c) {
  (void)o;
  (void)root;
  (void)c;
  return copy_buf(s, r, n, t);
}
int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)o;
  (void)c;
  return copy_buf(s, r, n, t);
}
int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int rn, MPI_Datatype rt,
                  MPI_Comm c) {
  (void)rn;
  (void)rt;
  (void)c;
  return copy_buf(s, r, n, t);
}
int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int rn, MPI_Datatype rt, int root,
               MPI_Comm c) {
  (void)rn;
  (void)rt;
  (void)root;
  (void)c;
  return copy_buf(s, r, n, t);
}
int MPI_Scatterv(const void *s, const int *cnt, const int *disp, MPI_Datatype t, void *r, int rn,
                 MPI_Datatype rt, int root, MPI_Comm c) {
  (void)rn;
  (void)rt;
  (void)root;
  (void)c;
  return copy_buf((const char *)s + (size_t)disp[0] * dt_size(t), r, cnt[0], t);
}
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b;
  (void)n;
  (void)t;
  (void)root;
  (void)c;
  return 0;
}
int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c) {
  (void)b, (void)n, (void)t, (void)d, (void)g, (void)c;
  return p2p("MPI_Send");
}
int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Status *st) {
  (void)b, (void)n, (void)t, (void)s, (void)g, (void)c, (void)st;
  return p2p("MPI_Recv");
}
int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c, MPI_Request *q) {
  (void)b, (void)n, (void)t, (void)d, (void)g, (void)c, (void)q;
  return p2p("MPI_Isend");
}
int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Request *q) {
  (void)b, (void)n, (void)t, (void)s, (void)g, (void)c, (void)q;
  return p2p("MPI_Irecv");
}
int MPI_Wait(MPI_Request *q, MPI_Status *s) {
  (void)q;
  (void)s;
  return 0;
}
int MPI_Waitall(int n, MPI_Request *q, MPI_Status *s) {
  (void)n;
  (void)q;
  (void)s;
  return 0;
}
int MPI_Get_count(const MPI_Status *s, MPI_Datatype t, int *n) {
  (void)s;
  (void)t;
  *n = 0;
  return 0;
}
int MPI_Get_address(const void *p, MPI_Aint *a) {
  *a = (MPI_Aint)p;
  return 0;
}
int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *d, const MPI_Datatype *t,
                           MPI_Datatype *nt) {
  (void)n, (void)bl, (void)d, (void)t;
  *nt = 0;
  return 0;
}
int MPI_Type_commit(MPI_Datatype *t) {
  (void)t;
  return 0;
}
int MPI_Type_free(MPI_Datatype *t) {
  (void)t;
  return 0;
}
int MPI_Type_size(MPI_Datatype t, int *s) {
  *s = (int)dt_size(t);
  return 0;
}
int MPI_Type_get_extent(MPI_Datatype t, MPI_Aint *lb, MPI_Aint *ext) {
  *lb = 0;
  *ext = (MPI_Aint)dt_size(t);
  return 0;
}
