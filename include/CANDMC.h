/*
 * CANDMC.h for the GB300 QR hot path: the QR part of the reference's
 * umbrella header (include/CANDMC.h:19-32), with the single-GPU drop-in
 * declarations, and the eigensolver's full -> band reduction that calls the
 * 2D QR.  The MM and LU parts and the rest of SE are not provided by this
 * library.
 */
#ifndef __CANDMC_H__
#define __CANDMC_H__

/* binary tree TSQR on panels of matrices */
#include "candmc/bitree_tsqr.h"

/* TSQR with Householder vector reconstruction */
#include "candmc/hh_recon.h"

/* 2D QR algorithms for full matrices */
#include "candmc/qr_2d.h"

/* 2D QR with Yamamoto's basis-kernel representation for full matrices */
#include "candmc/qr_y2d.h"

/* symmetric full -> band reduction over 2D QR (the reference's alg/SE/CANSE.h) */
#include "candmc/full_to_band.h"

/* tau from Householder vectors (the reference's alg/shared/util.h) */
#include "candmc/util.h"

/* the C ABI underneath */
#include "candmc_gb300.h"

#endif
