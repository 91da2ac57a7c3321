/*
 * frontend_port.c - TEST INFRASTRUCTURE: CPU restatement of the findROI and
 * gaussMLE front end.  (Filled in below the sampler work.)
 */
#include "oracle.h"

int oracle_findroi_filter(float *frames, int ysize, int xsize, int zsize, double sigma1,
                          double sigma2, int boxsize, float minval, float *flags, int threads)
{
    (void)frames; (void)ysize; (void)xsize; (void)zsize; (void)sigma1; (void)sigma2;
    (void)boxsize; (void)minval; (void)flags; (void)threads;
    return BAMF_ERR_UNSUPPORTED;
}
int oracle_gaussmle_xynb(const float *rois, int sz, int nfits, float psf_sigma, int iterations,
                         float *params, float *crlb, float *loglik, int threads)
{
    (void)rois; (void)sz; (void)nfits; (void)psf_sigma; (void)iterations; (void)params;
    (void)crlb; (void)loglik; (void)threads;
    return BAMF_ERR_UNSUPPORTED;
}
int oracle_gaussmle_xynb_f64(const float *rois, int sz, int nfits, double psf_sigma,
                             int iterations, double *params, double *crlb, double *loglik,
                             int threads)
{
    (void)rois; (void)sz; (void)nfits; (void)psf_sigma; (void)iterations; (void)params;
    (void)crlb; (void)loglik; (void)threads;
    return BAMF_ERR_UNSUPPORTED;
}
