/*
 * Single-GPU stand-in for CANDMC's alg/shared/comm.h: the communicator and
 * 2D-grid view types keep the reference's members (comm.h:32-63, 66-84) so a
 * CANDMC caller compiles unchanged, but no MPI is involved.  On one GPU the
 * process grid is 1 x 1: every communicator has np = 1 and rank = 0, and the
 * QR entry points reject other views with CANDMC_ERR_ARG (reported through
 * candmc_dropin_last_status()) instead of calling MPI_Abort.
 */
#ifndef CANDMC_DROPIN_COMM_H
#define CANDMC_DROPIN_COMM_H

#include <stdint.h>

typedef int MPI_Comm;   /* opaque handle; only MPI_COMM_WORLD exists */
#ifndef MPI_COMM_WORLD
#define MPI_COMM_WORLD 0
#endif
typedef int64_t long_int;

typedef class CommData {
 public:
  MPI_Comm cm;
  int np;
  int rank;
  int color;
  int alive;
} CommData_t;

class pview {
 public:
  int rrow;          /* current root row */
  int rcol;          /* current root column */
  CommData_t crow;   /* row communicator */
  CommData_t ccol;   /* column communicator */
  CommData_t cdiag;  /* diagonal communicator */
  CommData_t cworld; /* world communicator */
};

#define SET_COMM(_cm, _rank, _np, _cdt) \
  do {                                  \
    (_cdt).cm = (_cm);                  \
    (_cdt).rank = (_rank);              \
    (_cdt).np = (_np);                  \
    (_cdt).alive = 1;                   \
    (_cdt).color = 0;                   \
  } while (0)

/* A 1 x 1 grid view (all communicators single-rank, roots at 0). */
inline pview candmc_single_gpu_view() {
  pview pv;
  pv.rrow = 0;
  pv.rcol = 0;
  SET_COMM(MPI_COMM_WORLD, 0, 1, pv.crow);
  SET_COMM(MPI_COMM_WORLD, 0, 1, pv.ccol);
  SET_COMM(MPI_COMM_WORLD, 0, 1, pv.cdiag);
  SET_COMM(MPI_COMM_WORLD, 0, 1, pv.cworld);
  return pv;
}

/* Status of the last drop-in call on this thread (CANDMC_OK or an error of
 * include/candmc_gb300.h); the reference's functions return void. */
int candmc_dropin_last_status(void);

#endif
