/*
 * Drop-in declaration of the reference's tau_recon (alg/shared/util.h:675-680),
 * same signature: tau from the Householder vectors in Y, which the reference's
 * tree code (construct_tsqr_Q.cxx:183, apply_tsqr_QT.cxx:137) and its tests
 * (test/QR/test_hh_recon.cxx:126) call.  Host pointers; the work runs on the
 * current CUDA device.
 */
#ifndef CANDMC_DROPIN_UTIL_H
#define CANDMC_DROPIN_UTIL_H

/* structure 'R' (whole columns), 'L' (below the diagonal), 'U' (rows 0..i) */
void tau_recon(const char structure, const int ncol, const int nrow, const int lda, double const* Y,
               double* tau);

#endif
