/*
 * Drop-in declaration of CANDMC's symmetric full -> band reduction
 * (alg/SE/CANSE.h:17-22), same signature.  Host pointers; the work runs on
 * the current CUDA device.  The grid view must be 1 x 1 (it stays so: the
 * reference's root rotations are taken modulo the grid size).  The form of
 * the panel CAQR's trailing updates is chosen with
 * candmc_dropin_set_precision (default: CANDMC_PREC_FP64).
 */
#ifndef CANDMC_DROPIN_FULL_TO_BAND_H
#define CANDMC_DROPIN_FULL_TO_BAND_H

#include "comm.h"

/* CANSE.h:17-22: A (n x n, lower triangle) -> band of width b in place */
void sym_full2band(double* A, int64_t lda_A, int64_t n, int64_t b, int64_t b_sub, pview* pv);

#endif
