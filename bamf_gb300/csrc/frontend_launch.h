/*
 * frontend_launch.h - gaussMLE launch shared by the FindROI translation
 * unit, for the pinned front end that fits each chunk's ROIs while later
 * chunks are still being copied (not part of the C-ABI).
 */
#ifndef BAMF_FRONTEND_LAUNCH_H
#define BAMF_FRONTEND_LAUNCH_H

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "bamf.h"

/* the largest fit window gaussMLE takes (IMSZBIG of the reference's
 * definitions.h) */
constexpr int GAUSS_MLE_MAX_SIZE = 21;

/* kernel_MLEFit_XYNB_ (CCD) of ROIs [range[0], min(range[1], capacity)) of
 * `rois` (sz x sz each, device), the range read on the device when the
 * kernel runs: parameter k of ROI i to params[stride * k + i] and crlb
 * alike, the log-likelihood to loglik[i].  `blocks` CTAs of 16 fits each,
 * grid-stride over the range. */
bamf_status launch_gauss_mle_range(const float *rois, int sz, float psf_sigma, int iterations, float *params,
                                   float *crlb, float *loglik, int64_t stride, const int64_t *range,
                                   int64_t capacity, int blocks, cudaStream_t stream);

#endif
