/*
 * Drop-in declarations of CANDMC's 2D QR entry points
 * (alg/QR/qr_2d/qr_2d.h), same signatures and defaults.  Host pointers; the
 * work runs on the current CUDA device.  The grid view must be 1 x 1; like
 * the reference, QR_2D and QR_2D_pipe advance pv->rrow / pv->rcol (modulo
 * the grid size, i.e. they stay 0) and QR_2D_2D works on a copy.  The
 * arithmetic form of the trailing update is chosen with
 * candmc_dropin_set_precision (default: CANDMC_PREC_FP64).
 */
#ifndef CANDMC_DROPIN_QR_2D_H
#define CANDMC_DROPIN_QR_2D_H

#include "bitree_tsqr.h"
#include "comm.h"
#include "hh_recon.h"

/* qr_2d.h:25-31 */
void compute_invT_from_Y(double const* Y, int64_t lda_Y, double* T, int64_t lda_T, int64_t mb,
                         int64_t b, pview* pv);

/* qr_2d.h:47-56 */
void compute_invT_from_Y(double const* Y1, int64_t lda_Y1, double const* Y2, int64_t lda_Y2,
                         double* T, int64_t lda_T, int64_t mb, int64_t b1, int64_t b2, pview* pv);

/* qr_2d.h:74-85 */
void update_A(double const* Y, int64_t lda_Y, double* A, int64_t lda_A, int64_t m, int64_t k,
              int64_t b, double const* W, pview* pv, double* aggreg_Y, int64_t lda_aY,
              bool W_is_T = false);

/* qr_2d.h:99-108 */
void upd_A(double const* Ybuf, int64_t lda_Y, double* A, int64_t lda_A, int64_t mb, int64_t kb,
           int64_t b, double const* W, pview* pv, bool W_is_T = false);

/* qr_2d.h:124-131 */
void QR_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, pview* pv, double* aggreg_Y,
           int64_t lda_aY);

/* qr_2d.h:293-302 */
void QR_2D_pipe(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, pview* pv,
                double* last_Y = NULL, int64_t lda_lY = 0, double* last_W = NULL,
                double* my_last_W = NULL);

/* qr_2d.h:176-188 */
void QR_2D_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, int64_t b_sub, pview* pv,
              double* aggreg_Y, int64_t lda_aY, int* desc_A = NULL, double* org_A = NULL,
              int64_t IA = 1, int64_t JA = 1);

/* trailing-update arithmetic of the drop-in 2D QR (no counterpart in the reference) */
void candmc_dropin_set_precision(int precision);

#endif
