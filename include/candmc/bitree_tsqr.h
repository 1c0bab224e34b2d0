/*
 * Drop-in declarations of CANDMC's TSQR entry points
 * (alg/QR/tsqr/bitree_tsqr.h), same signatures and defaults.  Pointers are
 * host memory as in the reference; the work runs on the current CUDA device.
 * With numPes == 1 (the only grid one GPU has) the binary tree of the
 * reference is the single-rank path: bitree_tsqr = dgeqrf of the panel
 * (bitree_tsqr.cxx:129-146), construct_Q1 = dorgqr (construct_tsqr_Q.cxx:87-96),
 * apply_tsqr_QT = Q^T B (apply_tsqr_QT.cxx:31-163 at one rank).
 */
#ifndef CANDMC_DROPIN_BITREE_TSQR_H
#define CANDMC_DROPIN_BITREE_TSQR_H

#include "comm.h"

#ifndef TAU_BLK
#define TAU_BLK 16
#endif

/* bitree_tsqr.h:18-21: QR of [R1; R2] (2b x b, ld 2b); A becomes R over V,
 * tau (if not NULL) receives the b x min(b, TAU_BLK) block-diagonal T. */
void tree_tsqr(double* A, double* buf, int64_t const b, double* tau = NULL);

/* bitree_tsqr.h:33-38: Householder QR of one m x b block (dgeqrf). */
void local_tsqr(double* A, double* R, int64_t const m, int64_t const b, int64_t const lda_A,
                double* tau = NULL);

/* bitree_tsqr.h:58-70 */
void bitree_tsqr(double* A, int64_t const lda_A, double* R, double* tau, int64_t const m,
                 int64_t const b, int64_t const myRank, int64_t const numPes, int64_t const root,
                 int64_t const req_id, CommData_t cdt, int64_t const output_Y = 0,
                 double* tree_data = NULL);

/* bitree_tsqr.h:91-104 */
void construct_Q1(double const* Y, int64_t const lda_Y, double const* tau, double* Q1,
                  int64_t const lda_Q, int64_t const m, int64_t const b, int64_t const k,
                  int64_t const myRank, int64_t const numPes, int64_t const root, CommData_t cdt,
                  double* tree_data = NULL, double* ID = NULL);

/* bitree_tsqr.h:126-138 */
void apply_tsqr_QT(double const* Y, int64_t const lda_Y, double const* tau, double* B,
                   int64_t const lda_B, int64_t const m, int64_t const b, int64_t const k,
                   int64_t const myRank, int64_t const numPes, int64_t const root, CommData_t cdt,
                   double* tree_data = NULL);

#endif
