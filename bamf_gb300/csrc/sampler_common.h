/*
 * sampler_common.h - device-side data layout shared by the sampler kernels
 * and their host launcher.
 */
#ifndef BAMF_SAMPLER_COMMON_H
#define BAMF_SAMPLER_COMMON_H

#include <stdint.h>

#include "bamf.h"

namespace bamf {

/* A prior table after the reference's Stat construction
 * (source/c/LibRJMCMC.cpp:176-217): grid x[L] and pdf[L] for findPDF,
 * unique CDF uc[nu] and its grid ux[nu] for genRand. */
struct DevStat {
    const float *x;
    const float *pdf;
    const float *ux;
    const float *uc;
    int L;
    int nu;
    float inv_dx; /* 1 / grid step (fast-arithmetic lookups) */
};

/* Everything uniform over a batch of chains. */
struct SamplerConsts {
    bamf_mcmc_params p;
    float PVB[8];   /* cumulative P_Burnin (cRJMCMC.cpp:37-47) */
    float PVT[8];   /* cumulative P_Trials                      */
    DevStat off, sig, back;
    uint32_t seed;
    float bg0;      /* starting BG when no per-ROI start state is given */
    int32_t sync_moves; /* fast mode: CTA-synchronous move choice (rjmcmc_kernel_sync) */
    int32_t proposal;   /* BAMF_PROPOSAL_* (fast mode only) */
    int32_t opt_model;  /* 0 Gaussian PSF, 1 sampled PSF (p.PSFsize, SamplerBatch::sampled_psf) */
};

/* Per-ROI inputs and outputs of a batch.  Arrays indexed by ROI id. */
struct SamplerBatch {
    int n_rois;
    int side_max;                 /* max(xsize, ysize) over the batch      */
    const float *data;            /* ROI pixels, column-major, y fastest   */
    const int64_t *offsets;       /* pixel offset of each ROI in data      */
    const int32_t *xsize;
    const int32_t *ysize;
    const float *psf_sigma;       /* per-ROI sigma, or null: p.PSFsigma    */
    const float *scmos;           /* same layout as data, or null: zeros   */
    const int32_t *order;         /* work-queue order (ROI ids), or null   */
    /* optional start states: n, then BG, then I/X/Y rows of BAMF_NMAX */
    const int32_t *init_n;
    const float *init_bg;
    const float *init_ixy;        /* [roi][3][BAMF_NMAX]                   */
    const uint32_t *chain_ids;    /* Philox chain id per ROI, or null: id  */
    const uint32_t *rng_offset;   /* first stream index per ROI, or null   */
    /* outputs (any may be null) */
    int32_t *final_n;             /* [roi]                                 */
    float *final_state;           /* [roi][4 + 4*BAMF_NMAX]: BG ABG BBG -, I[], X[], Y[], S[] */
    int32_t *counters;            /* [roi][30] bamf_counters order          */
    uint8_t *nsig_trace;          /* [roi][trace_cap] Signal==1 count per entry */
    int32_t trace_cap;
    float *x_trace;               /* [roi][x_cap] mean X of the Signal==1 emitters */
    int32_t x_cap;
    const float *sampled_psf;     /* OptModel 1: n_psf sampled PSFs, one after another */
    const int32_t *psf_slot;      /* [roi] which of them, or null: the first */
    int32_t n_psf;
    const float *birth_cdf;       /* learned birth density (bamf_roi_batch)  */
    const float *birth_sub;
    int32_t *n_entries;           /* [roi] recorded chain entries          */
    uint32_t *uniforms_used;      /* [roi]                                 */
    int32_t *status;              /* [roi] 0 ok, else BAMF_ERR_*           */
    int32_t *overflow;            /* [roi] proposals rejected at BAMF_NMAX */
    int32_t *llr_evals;           /* [roi] likelihood-ratio evaluations     */
    float *model_drift;           /* [roi] largest relative model drift at the periodic rebuilds (fast) */
    float *pgrid;                 /* [slot][grid_stride] or null           */
    float *pback;
    int64_t grid_stride;
    int32_t grid_ld;              /* column stride of a grid; 0: the ROI's zoomed height */
    const int32_t *grid_slot;     /* grid of each ROI, or null: the ROI's own */
    float *pos_trace;             /* [roi][pos_len][BAMF_POS_RECORD] thinned states */
    int32_t pos_len;
    int32_t pos_thin;
    /* full chain recording (exact cRJMCMC outputs), or null */
    bamf_chain *chains;           /* device array [roi][2] of bamf_chain with device pointers */
    int32_t *queue;               /* work-queue counter (device int)       */
    /* size-class scheduling: when class_range is set, this launch runs the
     * ROIs order[class_range[2c] .. class_range[2c+1]) of class c = cls */
    const int32_t *class_range;
    int32_t cls;
};

/* Size classes by ROI side: (0,8] (8,12] (12,16] (16,20] (20,24] (24,28] (28,32]. */
/* ROIs (consecutive slots of a size class) that share one move-type stream in
 * the move-synchronous fast kernel; a CTA holds at most this many chains. */
#define BAMF_SYNC_GROUP 24
#define BAMF_N_CLASSES 7
/* device bytes of the batch order of n ROIs: the order, the ids of its
 * first pass (4 bytes each) and the photon buckets (1 byte each) */
#define BAMF_ORDER_SCRATCH(n) ((size_t)(n) * 9 + 16)
__host__ __device__ inline int side_class(int side)
{
    return side <= 8 ? 0 : (side <= 12 ? 1 : (side <= 16 ? 2 : (side <= 20 ? 3 : (side <= 24 ? 4 : (side <= 28 ? 5 : 6)))));
}
__host__ __device__ inline int class_side(int c) { return c == 0 ? 8 : 8 + 4 * c; }

}  // namespace bamf

#endif
