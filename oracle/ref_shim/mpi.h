/* Single-process MPI for building the reference's QR sources as a CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference's QR path (alg/QR/..., alg/shared/
 * comm.h:6,16) includes "mpi.h" unconditionally, and the image has no MPI.
 * This header supplies the MPI subset those sources name, for a world of
 * exactly one rank: MPI_COMM_WORLD has size 1, every communicator split from
 * it is the same single rank, collectives are identities or copies (root ==
 * rank 0 == self), and point-to-point messages can only go to oneself, where
 * they are queued in a process-local mailbox matched by tag.  A receive that
 * finds no matching message aborts: on one rank that would be a deadlock.
 *
 * On one rank the reference's hot path reaches only Comm_rank/size/split,
 * Bcast, Allreduce, Reduce, Barrier and Wtime (bitree_tsqr.cxx:129-146 takes
 * the single-process branch; hh_recon.cxx:289,291; qr_2d.cxx:44,168,202,265).
 * Written for this project from the MPI 3.1 standard's C bindings.
 */
#ifndef CANDMC_ORACLE_MPI_SHIM_H
#define CANDMC_ORACLE_MPI_SHIM_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_bytes;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_COMM_NULL ((MPI_Comm)-1)
/* datatypes encode their size in bytes in the low byte */
#define MPI_CHAR ((MPI_Datatype)(0x100 | 1))
#define MPI_INT ((MPI_Datatype)(0x200 | 4))
#define MPI_LONG ((MPI_Datatype)(0x300 | 8))
#define MPI_LONG_LONG_INT ((MPI_Datatype)(0x400 | 8))
#define MPI_LONG_LONG ((MPI_Datatype)(0x400 | 8))
#define MPI_DOUBLE ((MPI_Datatype)(0x500 | 8))
#define MPI_FLOAT ((MPI_Datatype)(0x600 | 4))
#define MPI_DOUBLE_COMPLEX ((MPI_Datatype)(0x700 | 16))
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_REQUEST_NULL ((MPI_Request)0)

static inline size_t candmc_mpi_size(MPI_Datatype t) { return (size_t)(t & 0xff); }

static inline void candmc_mpi_fail(const char* what) {
  fprintf(stderr, "single-rank MPI shim: %s\n", what);
  abort();
}

/* ---- self mailbox (point-to-point to rank 0 only) ---- */
typedef struct candmc_mpi_msg {
  int tag;
  size_t bytes;
  void* data;
  struct candmc_mpi_msg* next;
} candmc_mpi_msg;

static candmc_mpi_msg* candmc_mpi_box = 0;

static inline void candmc_mpi_post(const void* buf, size_t bytes, int tag) {
  candmc_mpi_msg* m = (candmc_mpi_msg*)malloc(sizeof(candmc_mpi_msg));
  m->tag = tag;
  m->bytes = bytes;
  m->data = malloc(bytes ? bytes : 1);
  if (bytes) memcpy(m->data, buf, bytes);
  m->next = 0;
  candmc_mpi_msg** p = &candmc_mpi_box;
  while (*p) p = &(*p)->next;
  *p = m;
}

static inline void candmc_mpi_take(void* buf, size_t cap, int tag, MPI_Status* st) {
  candmc_mpi_msg** p = &candmc_mpi_box;
  while (*p && !(tag == MPI_ANY_TAG || (*p)->tag == tag)) p = &(*p)->next;
  if (!*p) candmc_mpi_fail("receive with no matching message (deadlock on one rank)");
  candmc_mpi_msg* m = *p;
  if (m->bytes > cap) candmc_mpi_fail("message larger than the receive buffer");
  if (m->bytes) memcpy(buf, m->data, m->bytes);
  if (st) {
    st->MPI_SOURCE = 0;
    st->MPI_TAG = m->tag;
    st->MPI_ERROR = 0;
    st->count_bytes = (int)m->bytes;
  }
  *p = m->next;
  free(m->data);
  free(m);
}

static inline void candmc_mpi_check_rank(int r) {
  if (r != 0 && r != MPI_ANY_SOURCE) candmc_mpi_fail("peer rank != 0 on a one-rank world");
}

/* ---- environment ---- */
static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; fprintf(stderr, "MPI_Abort(%d)\n", code); abort(); return 0; }
static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Comm_size(MPI_Comm c, int* n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out) {
  (void)c; (void)color; (void)key; *out = MPI_COMM_WORLD; return 0;
}
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* out) { *out = c; return 0; }
static inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

/* ---- collectives on one rank ---- */
static inline int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm c) {
  (void)buf; (void)count; (void)t; (void)c; candmc_mpi_check_rank(root); return 0;
}
static inline int MPI_Allreduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  if (sb != MPI_IN_PLACE && count > 0) memmove(rb, sb, (size_t)count * candmc_mpi_size(t));
  return 0;
}
static inline int MPI_Reduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  candmc_mpi_check_rank(root);
  return MPI_Allreduce(sb, rb, count, t, op, c);
}
static inline int MPI_Scatter(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, int root, MPI_Comm c) {
  (void)c; (void)rc; (void)rt; candmc_mpi_check_rank(root);
  if (sb != MPI_IN_PLACE && rb != MPI_IN_PLACE && sc > 0) memmove(rb, sb, (size_t)sc * candmc_mpi_size(st));
  return 0;
}
static inline int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, int root, MPI_Comm c) {
  return MPI_Scatter(sb, sc, st, rb, rc, rt, root, c);
}
static inline int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, MPI_Comm c) {
  return MPI_Scatter(sb, sc, st, rb, rc, rt, 0, c);
}
static inline int MPI_Alltoall(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, MPI_Comm c) {
  return MPI_Scatter(sb, sc, st, rb, rc, rt, 0, c);
}
static inline int MPI_Scatterv(const void* sb, const int* sc, const int* sd, MPI_Datatype st, void* rb, int rc,
                               MPI_Datatype rt, int root, MPI_Comm c) {
  (void)c; (void)rc; (void)rt; candmc_mpi_check_rank(root);
  if (sc[0] > 0) memmove(rb, (const char*)sb + (size_t)sd[0] * candmc_mpi_size(st), (size_t)sc[0] * candmc_mpi_size(st));
  return 0;
}
static inline int MPI_Gatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int* rc, const int* rd,
                              MPI_Datatype rt, int root, MPI_Comm c) {
  (void)c; (void)rc; candmc_mpi_check_rank(root);
  if (sc > 0) memmove((char*)rb + (size_t)rd[0] * candmc_mpi_size(rt), sb, (size_t)sc * candmc_mpi_size(st));
  return 0;
}
static inline int MPI_Alltoallv(const void* sb, const int* sc, const int* sd, MPI_Datatype st, void* rb,
                                const int* rc, const int* rd, MPI_Datatype rt, MPI_Comm c) {
  (void)c; (void)rc;
  if (sc[0] > 0)
    memmove((char*)rb + (size_t)rd[0] * candmc_mpi_size(rt), (const char*)sb + (size_t)sd[0] * candmc_mpi_size(st),
            (size_t)sc[0] * candmc_mpi_size(st));
  return 0;
}

/* ---- point to point, self only ---- */
static inline int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c) {
  (void)c; candmc_mpi_check_rank(dest);
  candmc_mpi_post(buf, (size_t)count * candmc_mpi_size(t), tag);
  return 0;
}
static inline int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c, MPI_Request* r) {
  *r = MPI_REQUEST_NULL;
  return MPI_Send(buf, count, t, dest, tag, c);
}
static inline int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* st) {
  (void)c; candmc_mpi_check_rank(src);
  candmc_mpi_take(buf, (size_t)count * candmc_mpi_size(t), tag, st);
  return 0;
}
/* A nonblocking receive completes at once: the matching send to oneself must
 * already have been posted, as it must be on one rank. */
static inline int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request* r) {
  *r = MPI_REQUEST_NULL;
  return MPI_Recv(buf, count, t, src, tag, c, MPI_STATUS_IGNORE);
}
static inline int MPI_Wait(MPI_Request* r, MPI_Status* st) { (void)r; (void)st; return 0; }
static inline int MPI_Waitall(int n, MPI_Request* r, MPI_Status* st) { (void)n; (void)r; (void)st; return 0; }
static inline int MPI_Sendrecv(const void* sb, int sc, MPI_Datatype st, int dest, int stag, void* rb, int rc,
                               MPI_Datatype rt, int src, int rtag, MPI_Comm c, MPI_Status* status) {
  MPI_Send(sb, sc, st, dest, stag, c);
  return MPI_Recv(rb, rc, rt, src, rtag, c, status);
}

/* profiling-layer names (alg/shared/timer.cxx calls PMPI_* directly) */
#define PMPI_Allreduce MPI_Allreduce
#define PMPI_Reduce MPI_Reduce
#define PMPI_Bcast MPI_Bcast
#define PMPI_Send MPI_Send
#define PMPI_Recv MPI_Recv
#define PMPI_Barrier MPI_Barrier

#ifdef __cplusplus
}
#endif

#endif
