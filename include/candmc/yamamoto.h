/*
 * Drop-in declaration of CANDMC's Yamamoto panel factorization
 * (alg/QR/hh_recon/yamamoto.h:21-32), same signature.  Host pointers; the
 * work runs on the current CUDA device; numPes must be 1.  On return A holds
 * Y\(S*R) (Householder Y below the diagonal), Qm = [Q1 - S; Q2] and
 * W = (Q1 - S)^-1 S (b x b, ld b) for a TSQR basis [Q1; Q2]: the reference's
 * pair up to its own column signs, with the same Qm W Qm^T.
 */
#ifndef CANDMC_DROPIN_YAMAMOTO_H
#define CANDMC_DROPIN_YAMAMOTO_H

#include "comm.h"

void Yamamoto(double* A, int64_t lda_A, double* Qm, int64_t lda_Qm, int64_t m, int64_t b, double* W,
              int64_t myRank, int64_t numPes, int64_t root, int64_t req_id, CommData_t cdt);

#endif
