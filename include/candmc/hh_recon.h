/*
 * Drop-in declarations of CANDMC's Householder-reconstruction entry points
 * (alg/QR/hh_recon/hh_recon.h), same signatures.  Host pointers; the work
 * runs on the current CUDA device; numPes must be 1.
 */
#ifndef CANDMC_DROPIN_HH_RECON_H
#define CANDMC_DROPIN_HH_RECON_H

#include "comm.h"

/* hh_recon.h:13-15: invT holds Y1 on entry, T^-T = -W^-T Y1 on return. */
void compute_invT_from_W(double const* W, int64_t b, double* invT);

/* hh_recon.h:27-36 */
void signed_NLU(double* A, double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs);

/* hh_recon.h:38-49 */
void recursive_NLU(double* A, double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs);

/* hh_recon.h:66-75 */
void hh_recon_qr(double* A, int64_t lda_A, int64_t m, int64_t b, double* W, int64_t myRank,
                 int64_t numPes, int64_t root, int64_t req_id, CommData_t cdt);

#endif
