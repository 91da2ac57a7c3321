/*
 * oracle.h - TEST INFRASTRUCTURE: the CPU oracle, a plain-C restatement of
 * the reference algorithms on the BAMF hot path.  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg use it, as the checker; the product
 * never links it.
 *
 *   rjmcmc_port.c   RJMCMC sampler (source/c/LibRJMCMC.cpp + cRJMCMC.cpp set-up)
 *   frontend_port.c findROI kernels + glue (cuda_FindROI.cu, findROI.m) and
 *                   gaussMLE _XYNB_ (cuda_gaussMLEv2.cu, GPUgaussLib.cuh,
 *                   MatInvLib.h), in float and in double
 *
 * Parity status: the sampler port is pinned against the reference sampler
 * compiled from its own sources (oracle/_ref) and against golden fixtures
 * made from it (tests/golden/).
 */
#ifndef BAMF_ORACLE_H
#define BAMF_ORACLE_H

#include <stdint.h>
#include "bamf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sampler ---------------------------------------------------------- */
void *oracle_rjmcmc_run(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                        const bamf_mcmc_params *p, const float *off, int loff, const float *sig,
                        int lsig, const float *back, int lback, const float *scmos,
                        const bamf_rng *rng);
/* The same with cRJMCMC's last two inputs (cRJMCMC.cpp:73-74): the sampled
 * PSF (p->PSFsize extents, first index fastest) and OptModel (0 Gaussian,
 * 1 sampled PSF). */
void *oracle_rjmcmc_run_model(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                              const bamf_mcmc_params *p, const float *off, int loff, const float *sig,
                              int lsig, const float *back, int lback, const float *scmos,
                              const float *sampled_psf, int opt_model, const bamf_rng *rng);
int oracle_result_sizes(void *h, int64_t *sizes);
int oracle_result_chain(void *h, int which, bamf_chain *out);
int oracle_result_grids(void *h, float *pgrid, float *pback);
int oracle_result_counters(void *h, bamf_counters *c);
void oracle_result_free(void *h);

/* Batch of independent ROIs (same priors and parameters) on `threads` host
 * threads; per ROI it returns only the summary the GPU batch path returns:
 * the final state, the MAP emitter count of the chain's second half and the
 * acceptance counters.  sigma: per-ROI PSF sigma or NULL (p->PSFsigma).
 * Used as the CPU baseline. */
int oracle_rjmcmc_batch(const float *data, const int64_t *offsets, const int32_t *xs,
                        const int32_t *ys, const float *sigma, int n_rois, const bamf_mcmc_params *p,
                        const float *off, int loff, const float *sig, int lsig,
                        const float *back, int lback, float bg0, uint32_t seed, int threads,
                        int32_t *final_n, int32_t *map_n, int32_t *n_accepted);

/* ---- front end -------------------------------------------------------- */
int oracle_findroi_filter(float *frames, int ysize, int xsize, int zsize, double sigma1,
                          double sigma2, int boxsize, float minval, float *flags, int threads);
int oracle_findroi_dog(const float *frames, int ysize, int xsize, int zsize, double sigma1, double sigma2,
                       float *dog);
int oracle_gaussmle_xynb(const float *rois, int sz, int nfits, float psf_sigma, int iterations,
                         float *params, float *crlb, float *loglik, int threads);
int oracle_gaussmle_xynb_f64(const float *rois, int sz, int nfits, double psf_sigma,
                             int iterations, double *params, double *crlb, double *loglik,
                             int threads);

/* the parity math (include/bamf_parity_math.h) on the host: 0 erf, 1 log, 2 exp */
int oracle_parity_math(int fn, const float *x, int n, float *out);

#ifdef __cplusplus
}
#endif

#endif
