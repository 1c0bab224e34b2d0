/*
 * Drop-in declarations of CANDMC's 2D QR with Yamamoto's basis-kernel
 * representation (alg/QR/qr_2d/qr_y2d.h), same signatures and defaults.
 * Host pointers, including the aggregator's arrays; the work runs on the
 * current CUDA device.  The grid view must be 1 x 1.  The arithmetic form of
 * the trailing updates is chosen with candmc_dropin_set_precision.
 */
#ifndef CANDMC_DROPIN_QR_Y2D_H
#define CANDMC_DROPIN_QR_Y2D_H

#include <stddef.h>

#include "comm.h"
#include "yamamoto.h"

/* qr_y2d.h:4-44: the panels' Qm stacked in aQm (lda_aQm x lda_aT), each one
 * shift rows lower, and the block lower-triangular aT (lda_aT x lda_aT), so
 * that I + aQm aT aQm^T applies the panels in order.  The arrays are host
 * memory, zeroed by the constructor and by reset. */
class aggregator {
 public:
  int64_t lda_aQm;
  int64_t lda_aT;
  int64_t shift;
  double* aQm;
  double* aT;
  int64_t n;

  aggregator(int64_t lda_aQm, int64_t lda_aT);
  ~aggregator();
  void reset();
  void shift_down(int64_t b);
  void append(int64_t mb, int64_t b, double const* Qm, int64_t lda_Qm, double const* T, pview* pv);
};

/* qr_y2d.h:58-68: (I + Qm T Qm^T) A, appending Qm and T to agg when non-null */
void update_Yamamoto_A(double* Qm, int64_t lda_Qm, double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b,
                       double* T, pview* pv, aggregator* agg);

/* qr_y2d.h:84-92 */
void upd_Yamamoto_A(double const* Qm, int64_t lda_Qm, double* A, int64_t lda_A, int64_t mb, int64_t kb,
                    int64_t b, double const* T, pview* pv);

/* qr_y2d.h:106-113 */
void QR_Yamamoto_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, pview* pv,
                    aggregator* agg = NULL, bool compute_Y = false);

/* qr_y2d.h:129-137 */
void QR_Yamamoto_2D_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, int64_t b_sub, pview* pv,
                       aggregator* agg = NULL, bool compute_Y = false);

#endif
