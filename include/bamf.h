/*
 * bamf.h - C ABI of the GB300-native BAMF hot path (libbamf_gb300.so).
 *
 * Three groups of entry points, each replacing one reference interface:
 *   - the reversible-jump sampler   (MEX cRJMCMC, source/c/cRJMCMC.cpp:52-308)
 *   - the ROI finder                (findROI, @RJ/findROI.m:1-224 driving
 *                                    source/cuda/cuda_FindROI/cuda_FindROI.cu)
 *   - the single-emitter MLE fitter (gaussMLE, @RJ/gaussMLE.m:64-211 driving
 *                                    kernel_MLEFit_XYNB_, cuda_gaussMLEv2.cu:16-141)
 * (bamf_find_roi_fit_pinned runs the last two as one pipelined call on
 * frames in pinned host memory.)
 *
 * Conventions: plain C types only; every function returns a bamf_status;
 * images are column-major with y (MATLAB rows) fastest, exactly as MATLAB
 * hands them to a MEX file: pixel (y, x) of a Ysize x Xsize image lives at
 * y + x * Ysize.  "_host" entry points take host pointers and copy in and
 * out themselves; "_device" entry points take device pointers and a CUDA
 * stream (cudaStream_t passed as void*), enqueue work and return without
 * synchronising.  Nothing here is thread-safe across calls that share a
 * bamf_workspace.
 */
#ifndef BAMF_H
#define BAMF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int bamf_status;
#define BAMF_OK 0
#define BAMF_ERR_INVALID_ARG 1   /* null pointer, bad size, bad enum         */
#define BAMF_ERR_CUDA 2          /* a CUDA runtime call failed               */
#define BAMF_ERR_NO_DEVICE 3     /* no CUDA device visible                   */
#define BAMF_ERR_TOO_LARGE 4     /* size beyond a documented kernel limit    */
#define BAMF_ERR_TIMEOUT 5       /* a bounded device wait ran out            */
#define BAMF_ERR_BAD_PRIOR 6     /* prior PDF table not usable (NaN, <0, ...)*/
#define BAMF_ERR_CAPACITY 7      /* caller-provided output buffer too small  */
#define BAMF_ERR_UNSUPPORTED 8   /* option not implemented (e.g. OptModel=1) */

/* Largest emitter count a GPU chain state can hold.  A proposal that would
 * exceed it is rejected and counted in bamf_chain_summary.overflow. */
#define BAMF_NMAX 32
/* Largest ROI side the sampler kernels accept (pixels). */
#define BAMF_MAX_ROI_SIDE 32

/* Move-type codes recorded in the chain (the reference's JumpType values,
 * LibRJMCMC.cpp:757-787,849,974,1113,1260,1334,1391,1488). */
#define BAMF_JT_JUMP 1
#define BAMF_JT_BG 2
#define BAMF_JT_GROUP 3
#define BAMF_JT_SPLIT 4
#define BAMF_JT_MERGE 5
#define BAMF_JT_BIRTH 6
#define BAMF_JT_DEATH 7
#define BAMF_JT_GSPLIT 8
#define BAMF_JT_GMERGE 9
#define BAMF_JT_GROUP_CONSERVE 10

/*
 * Sampler parameters: the MATLAB struct `MCMC` that rjmcmc.m:49-78 builds
 * and make_Params (cRJMCMC.cpp:14-50) unpacks into MCMC_Parameters
 * (LibRJMCMCreturn.hpp:33-56), field for field.  P_Burnin/P_Trials are the
 * raw 8-slot move probabilities [jump, split, merge, birth, death, gSplit,
 * gMerge, backFore]; the library forms the cumulative PV_* vectors itself.
 */
typedef struct bamf_mcmc_params {
    float PSFsigma;
    int32_t N_Trials;
    int32_t N_Burnin;
    float I_stdFg, I_stdBg;
    float X_stdFg, X_stdBg;
    float P_Burnin[8];
    float P_Trials[8];
    float Rho;
    float Bnd_out;
    int32_t Grid_Zoom;
    float Split_std;
    float Icutoff;
    float BG_std;
    float ABBG_std;
    float DX;
    float DriftX, DriftY;
    int32_t PSFsize[4];
    int32_t IsBackg;
} bamf_mcmc_params;

/* Starting state: the MATLAB struct `E_active` (rjmcmc.m:43-47). */
typedef struct bamf_emitters {
    int32_t N;
    const float *I;
    const float *X;
    const float *Y;
    float BG;
} bamf_emitters;

/* Uniform stream of a chain: Philox4x32-10 keyed (seed, chain_id); the
 * chain starts at value index `offset` (include/bamf_philox.h). */
typedef struct bamf_rng {
    uint32_t seed;
    uint32_t chain_id;
    uint32_t offset;
} bamf_rng;

/* Arithmetic of a sampler run.
 *   BAMF_ARITH_EXACT: the reference's float operation order, serial pixel
 *     sums and the project's parity erf/log/exp; reproduces the parity build
 *     of the reference sampler bit for bit.
 *   BAMF_ARITH_FAST: hardware SFU math, incremental model updates and
 *     warp-tree reductions; same moves and acceptance rule, not bitwise. */
#define BAMF_ARITH_EXACT 0
#define BAMF_ARITH_FAST 1

/*
 * Recorded chain: the raw vectors of RJMCMCChain (LibRJMCMCreturn.hpp:119-153).
 * Per entry (one per recorded proposal): N, LLR, PR, JumpType, Accepted, BG,
 * ABG, BBG.  Per emitter record: Index (1-based entry number), Photons, X, Y,
 * Signal; an entry with no emitters holds one placeholder record
 * (Photons 0, X = Y = -100, Signal -1; LibRJMCMC.cpp:306-314).
 * The caller allocates every array with the capacities it states; the
 * library fills n_entries / n_records.  Capacities of (N_Burnin + N_Trials)
 * entries and (N_Burnin + N_Trials) * BAMF_NMAX records always suffice.
 */
typedef struct bamf_chain {
    int32_t capacity_entries;
    int32_t capacity_records;
    int32_t n_entries;
    int32_t n_records;
    int32_t *N;
    float *LLR;
    float *PR;
    int32_t *JumpType;
    int32_t *Accepted;
    float *BG;
    float *ABG;
    float *BBG;
    int32_t *Index;
    float *Photons;
    float *X;
    float *Y;
    int32_t *Signal;
} bamf_chain;

/* The 30 proposal/accept counters of class RJMCMC (LibRJMCMCreturn.hpp:192-197),
 * initialised like LibRJMCMC.cpp:672-677 (N_* = 1, A_* = 0). */
typedef struct bamf_counters {
    int32_t N_jump, N_split, N_merge, N_birth, N_death;
    int32_t A_jump, A_split, A_merge, A_birth, A_death;
    int32_t N_jumpFg, N_splitFg, N_mergeFg, N_birthFg, N_deathFg;
    int32_t A_jumpFg, A_splitFg, A_mergeFg, A_birthFg, A_deathFg;
    int32_t N_jumpBg, N_splitBg, N_mergeBg, N_birthBg, N_deathBg;
    int32_t A_jumpBg, A_splitBg, A_mergeBg, A_birthBg, A_deathBg;
} bamf_counters;

/* ------------------------------------------------------------------ */
/* Library                                                              */
/* ------------------------------------------------------------------ */

/* Version string of the library. */
const char *bamf_version(void);

/* Number of visible CUDA devices (0 when none; never fails). */
int bamf_device_count(void);

/* Text of the last CUDA error this thread's calls met (empty if none). */
const char *bamf_last_error(void);

/* ------------------------------------------------------------------ */
/* Sampler                                                              */
/* ------------------------------------------------------------------ */

/*
 * One ROI with the exact semantics of the MEX function cRJMCMC
 * (source/c/cRJMCMC.cpp:52-308; called from @RJ/rjmcmc.m:102 and
 * @RJ/mcmc.m:142).  Host buffers in, host buffers out; synchronous.
 *
 *   data            Ysize*Xsize floats, y fastest            (prhs[0])
 *   xsize, ysize                                             (prhs[3], prhs[4])
 *   e0              starting emitters and offset             (prhs[1])
 *   p               the MCMC struct                          (prhs[2])
 *   off/sig/back    OffSetPDF, SignalPDF, BackPDF and lengths (prhs[5..7];
 *                   length = max(dims) as the gateway takes it, :77-98)
 *   scmos           Ysize*Xsize sCMOS variance image or NULL (zeros)  (prhs[8])
 *   rng             the chain's uniform stream (stands in for rand())
 *   arith           BAMF_ARITH_EXACT or BAMF_ARITH_FAST
 *   pgrid, pback    (Ysize*Zoom)*(Xsize*Zoom) floats, y fastest; may be
 *                   NULL together                            (plhs[0], plhs[1])
 *   chain, chain_test  raw RJMCMCChain vectors (see bamf_chain); may be NULL
 *                   (plhs[2], plhs[3] before marshalling)
 *   counters        the 30 counters behind the Stat output  (plhs[4]); may be NULL
 *
 * This entry point uses the Gaussian PSF (OptModel 0); the sampled-PSF
 * model (prhs[9], prhs[10] = OptModel 1) is bamf_crjmcmc_host_model.
 * Errors: BAMF_ERR_INVALID_ARG (null input, size < 1, pdf length < 1),
 * BAMF_ERR_TOO_LARGE (side > BAMF_MAX_ROI_SIDE or N > BAMF_NMAX),
 * BAMF_ERR_BAD_PRIOR (NaN/negative pdf, non-increasing grid),
 * BAMF_ERR_CAPACITY (chain arrays too small), BAMF_ERR_CUDA, BAMF_ERR_NO_DEVICE.
 */
bamf_status bamf_crjmcmc_host(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                              const bamf_mcmc_params *p, const float *off, int off_len,
                              const float *sig, int sig_len, const float *back, int back_len,
                              const float *scmos, const bamf_rng *rng, int arith, float *pgrid,
                              float *pback, bamf_chain *chain, bamf_chain *chain_test,
                              bamf_counters *counters);

/* cRJMCMC with its last two inputs (cRJMCMC.cpp:73-74): sampled_psf
 * (host, bamf_mcmc_params.PSFsize extents) and opt_model (0 Gaussian PSF,
 * 1 the sampled PSF; sampled_psf may be NULL for 0).  bamf_crjmcmc_host is
 * this call with opt_model 0. */
bamf_status bamf_crjmcmc_host_model(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                                    const bamf_mcmc_params *p, const float *off, int off_len,
                                    const float *sig, int sig_len, const float *back, int back_len,
                                    const float *scmos, const float *sampled_psf, int opt_model,
                                    const bamf_rng *rng, int arith, float *pgrid, float *pback,
                                    bamf_chain *chain, bamf_chain *chain_test, bamf_counters *counters);

/* Prior PDF tables of a batch (host pointers; the library builds the
 * reference's CDF tables from them, LibRJMCMC.cpp:176-217). */
typedef struct bamf_priors {
    const float *offset_pdf;
    int32_t offset_len;
    const float *signal_pdf;
    int32_t signal_len;
    const float *back_pdf;
    int32_t back_len;
} bamf_priors;

/*
 * Many cRJMCMC calls in one launch: the per-ROI loop of analyzeROIs.m:126-159
 * (each iteration rjmcmc.m:102 -> MEX cRJMCMC, cRJMCMC.cpp:52-308) with the
 * full per-call outputs of bamf_crjmcmc_host for every ROI.  Host buffers,
 * synchronous; Gaussian PSF (OptModel 0).
 *   n_rois, data, offsets, xsize, ysize   ROI k at data[offsets[k]], y fastest
 *   e0          [n_rois] start states (prhs[1] of each call)
 *   p, priors   shared by all ROIs (prhs[2], prhs[5..7])
 *   scmos       laid out like data, or NULL (zeros)
 *   seed, chain_id[k] (NULL: k), rng_offset[k] (NULL: 0)  ROI k's uniform
 *               stream, as bamf_rng {seed, chain_id, offset}
 *   pgrids, pbacks  ROI k's (Ysize*Zoom)*(Xsize*Zoom) grid at
 *               Zoom*Zoom*offsets[k]; may be NULL together
 *   chains      [n_rois][2] (Chain, Chain_Test) with the caller's capacities,
 *               or NULL
 *   counters    [n_rois] or NULL;  uniforms_used [n_rois] uniforms each
 *               chain drew, or NULL
 *   status      [n_rois]: BAMF_OK, or that ROI's error (BAMF_ERR_CAPACITY
 *               when its chain arrays were too small; its outputs are then
 *               not written)
 * Errors of the call itself as bamf_crjmcmc_host.
 */
bamf_status bamf_crjmcmc_batch_host(int n_rois, const float *data, const int64_t *offsets,
                                    const int32_t *xsize, const int32_t *ysize, const bamf_emitters *e0,
                                    const bamf_mcmc_params *p, const bamf_priors *priors, const float *scmos,
                                    uint32_t seed, const uint32_t *chain_id, const uint32_t *rng_offset,
                                    int arith, float *pgrids, float *pbacks, bamf_chain *chains,
                                    bamf_counters *counters, uint32_t *uniforms_used, int32_t *status);

/*
 * A batch of independent ROIs of possibly different sizes, packed back to
 * back (the per-ROI calls of analyzeROIs.m:126-159 as one launch).
 * ROI k occupies data[offsets[k] .. offsets[k] + ysize[k]*xsize[k]), y fastest.
 * Optional arrays may be NULL: psf_sigma (then p->PSFsigma for all), scmos
 * (zeros), init_n/init_bg/init_ixy (empty start with BG = bg0, as
 * rjmcmc.m:43-47 does; init_ixy is [k][3][BAMF_NMAX] = I row, X row, Y row).
 * Pointers are device pointers for bamf_rjmcmc_batch_device and host
 * pointers for bamf_rjmcmc_batch_host.
 */
typedef struct bamf_roi_batch {
    int32_t n_rois;
    int32_t side_max;   /* largest ROI side in the batch; 0 = BAMF_MAX_ROI_SIDE */
    const float *data;
    const int64_t *offsets;
    const int32_t *xsize;
    const int32_t *ysize;
    const float *psf_sigma;
    const float *scmos;
    const int32_t *init_n;
    const float *init_bg;
    const float *init_ixy;
    float bg0;
    /* Birth proposal (fields past here may be left zero):
     *   BAMF_PROPOSAL_REFERENCE  the reference's: residual-weighted pixel,
     *                            position pixel + U - 0.5, its Hastings terms
     *                            (LibRJMCMC.cpp:1258-1387, 1688-1736)
     *   BAMF_PROPOSAL_UNIFORM    position uniform on the extended box
     *                            [-Bnd, X+Bnd] x [-Bnd, Y+Bnd] (Bnd = (int)Bnd_out),
     *                            intensity from SignalPDF; birth ratio
     *                            LLR * MeanN/(NEm+1) * P_death/P_birth and death
     *                            its inverse; raw phase probabilities in every
     *                            ratio; split/merge position prior 1/area of
     *                            the extended box, and the exact split/merge
     *                            pair accounting (the merge's pick of the pair,
     *                            both orderings of a split, unmergeable splits
     *                            rejected), which the reference's ratio omits
     *   BAMF_PROPOSAL_LEARNED    UNIFORM, with the birth position drawn half of
     *                            the time from a per-ROI density over 4x4
     *                            sub-cells of each pixel, half of the
     *                            splits placing the first emitter from that
     *                            density (intensity fraction triangular on
     *                            [0.3, 0.7]), and a quarter of the
     *                            single-emitter jumps relocating the emitter
     *                            to a position drawn from the birth mixture
     *                            (intensity kept); the exact mixture densities
     *                            enter the birth, death, split, merge and
     *                            relocation ratios
     * Anything but REFERENCE needs BAMF_ARITH_FAST.  LEARNED reads
     *   birth_cdf   [pixel] running sum of the pixel probabilities, laid out
     *               like data (ROI k at offsets[k], y fastest)
     *   birth_sub   [pixel][16] probabilities of the sub-cells of each pixel
     *               (sub-cell s = sy + 4*sx covers [x + sx/4, x + (sx+1)/4) x
     *               [y + sy/4, y + (sy+1)/4)), summing to 1 per pixel; ROI k
     *               at 16*offsets[k] */
    int32_t proposal;
    const float *birth_cdf;
    const float *birth_sub;
    /* Likelihood model (cRJMCMC.cpp:73-74, OptModel and SampledPSF):
     *   0  the Gaussian PSF of sigma psf_sigma / PSFsigma (Model, LibRJMCMC.cpp:15-59)
     *   1  the sampled PSF `sampled_psf` (NumModel, LibRJMCMC.cpp:67-170), one
     *      for the whole batch, of extents bamf_mcmc_params.PSFsize =
     *      [P0 y-pixels, P1 x-pixels, P2 y-sub-positions, P3 x-sub-positions],
     *      y fastest (MATLAB order); an emitter at (x, y) is centred on PSF
     *      pixel P0/2 and blends the sub-position planes floor(P3 * frac)
     *      and the next one bilinearly; a flat index outside the array reads
     *      its last element, as the reference does.
     * Several PSFs (analyzeROIs.m:142-146 uses one per sub-region position):
     * n_psf arrays one after another in sampled_psf, and psf_slot[k] the
     * one ROI k uses (NULL: all use the first; n_psf 0 counts as 1; a slot
     * outside [0, n_psf) sets that ROI's status to BAMF_ERR_INVALID_ARG).
     * sampled_psf and psf_slot are device pointers for the device entry
     * points, host pointers for bamf_rjmcmc_batch_host. */
    int32_t opt_model;
    const float *sampled_psf;
    int32_t n_psf;
    const int32_t *psf_slot;
} bamf_roi_batch;

#define BAMF_PROPOSAL_REFERENCE 0
#define BAMF_PROPOSAL_UNIFORM 1
#define BAMF_PROPOSAL_LEARNED 2

/* Per-ROI results of a batch (any pointer may be NULL).
 *   map_n        MAP emitter count: mode of the Signal==1 count over the
 *                second half of the accepted chain (findMap.m:29-45)
 *   final_n      emitters in the last state
 *   final_state  [k][4 + 4*BAMF_NMAX]: BG, ABG, BBG, N, I[], X[], Y[], Signal[]
 *   counters     [k][30] in bamf_counters order
 *   n_entries    recorded chain entries (cRJMCMC's chain length + 1)
 *   status       BAMF_OK or the ROI's error
 *   overflow     proposals rejected because they would exceed BAMF_NMAX
 *   llr_evals    likelihood-ratio evaluations (proposals scored against the
 *                data); each costs one pass over the ROI's pixels
 *   n_trace      [k][trace_len] Signal==1 emitter count of the accepted
 *                state at each chain entry (the first trace_len entries);
 *                with map_n it must hold N_Burnin + N_Trials entries
 *   x_trace      [k][trace_len] mean X of those emitters (NaN when none): a
 *                permutation-invariant position functional for ESS
 *   pgrid, pback posterior grids (update_grids, LibRJMCMC.cpp:1629-1648):
 *                each trial-phase step adds 1 at (round(Zoom (Y+DriftY)),
 *                round(Zoom (X+DriftX))) for every emitter with I > Icutoff,
 *                Signal==1 into pgrid, Signal==0 into pback (either may be
 *                NULL); grid g starts at g * grid_stride floats, column
 *                stride grid_ld (0: the ROI's Zoom*Ysize); ROI k writes grid
 *                grid_slot[k] (grid_slot NULL: grid k), so ROIs sharing a
 *                slot accumulate into one grid (the per-sub-region sum over
 *                frames of analyzeROIs.m:153).  The caller zeroes them.
 *   pos_trace    [k][pos_len][BAMF_POS_RECORD] thinned chain states: chain
 *                entry e = r * pos_thin is record r (r < pos_len): entry
 *                index, Signal==1 count, BG, ABG, BBG, then X, Y, I of up
 *                to BAMF_POS_SLOTS Signal==1 emitters in slot order (NaN
 *                past the count); the input of bamf_map_kmeans_device and
 *                bamf_refine_stats_device (findMap.m, mcmc.m)
 *   model_drift  [k] fast arithmetic only: the largest relative difference
 *                max_p |M_p - M'_p| / M'_p between the incrementally
 *                updated model image M and the model M' rebuilt from the
 *                chain's state, over the periodic rebuilds (every 512
 *                jumps); 0 when the chain had none.  No counterpart in the
 *                reference, which rebuilds the model for every proposal. */
typedef struct bamf_batch_results {
    int32_t *map_n;
    int32_t *final_n;
    float *final_state;
    int32_t *counters;
    int32_t *n_entries;
    int32_t *status;
    int32_t *overflow;
    int32_t *llr_evals;
    int32_t trace_len;
    uint8_t *n_trace;
    float *x_trace;
    float *pgrid;
    float *pback;
    int64_t grid_stride;
    int32_t grid_ld;
    const int32_t *grid_slot;
    float *pos_trace;
    int32_t pos_len;
    int32_t pos_thin;
    float *model_drift;
} bamf_batch_results;

#define BAMF_POS_SLOTS 32
#define BAMF_POS_RECORD (5 + 3 * BAMF_POS_SLOTS)

/* Chain summaries from pos_trace (device pointers; pos_trace as the batch
 * wrote it with pos_len <= 256 records of every pos_thin-th entry).  Output
 * per ROI: BAMF_MAP_RECORD floats = count, records used, Bg mean, Bg std,
 * ABg mean, BBg mean, then X, Y, I, X_SE, Y_SE, I_SE of BAMF_POS_SLOTS each
 * (NaN past the count).
 *   bamf_map_kmeans_device   findMap.m:29-111 (FB = 1): MAP count map_n
 *                            (from the full count trace, e.g. the batch's
 *                            map_n), then k-means of the positions of the
 *                            recorded second-half states with that count
 *                            and per-cluster mean / std (n-1) of X, Y, I
 *   bamf_refine_stats_device mcmc.m:142-169: per-emitter mean / std over
 *                            the recorded second half of a jumps-only chain
 */
#define BAMF_MAP_RECORD (6 + 6 * BAMF_POS_SLOTS)
bamf_status bamf_map_kmeans_device(const float *pos_trace, int pos_len, int pos_thin, const int32_t *n_entries,
                                   const int32_t *map_n, int n, int max_iter, float *out, void *stream);
bamf_status bamf_refine_stats_device(const float *pos_trace, int pos_len, int pos_thin, const int32_t *n_entries,
                                     int n, float *out, void *stream);

/* Device scratch (prior tables, work queue, per-ROI chain traces) that
 * grows on demand and is reused across calls on one stream; it also keeps
 * the CTA shapes chosen by bamf_autotune. */
typedef struct bamf_workspace bamf_workspace;
bamf_status bamf_workspace_create(bamf_workspace **ws);
void bamf_workspace_destroy(bamf_workspace *ws);

/* Batched sampler on device-resident data; enqueues on `stream`
 * (a cudaStream_t, NULL = default stream) and returns. */
bamf_status bamf_rjmcmc_batch_device(bamf_workspace *ws, const bamf_roi_batch *rois,
                                     const bamf_mcmc_params *p, const bamf_priors *priors,
                                     uint32_t seed, int arith, const bamf_batch_results *out,
                                     void *stream);

/* Same with host buffers: copies in, runs, copies out, synchronises. */
bamf_status bamf_rjmcmc_batch_host(bamf_workspace *ws, const bamf_roi_batch *rois,
                                   const bamf_mcmc_params *p, const bamf_priors *priors,
                                   uint32_t seed, int arith, const bamf_batch_results *out);

/* A batch as a CUDA graph (no reference counterpart): one run of the batch
 * on a private stream (which uploads the prior tables, sizes the workspace
 * and configures the kernels), then the same call captured into a graph:
 * the size-class ordering, every class's persistent launch (burn-in and
 * trial phases of all chains) on its forked stream, the MAP reduction.
 * Each launch replays it on the buffers named at creation (new data may be
 * written into them between launches; the seed is the one given here).
 * The workspace must not be used by other calls while the graph lives. */
typedef struct bamf_batch_graph bamf_batch_graph;
bamf_status bamf_rjmcmc_batch_graph_create(bamf_workspace *ws, const bamf_roi_batch *rois,
                                           const bamf_mcmc_params *p, const bamf_priors *priors, uint32_t seed,
                                           int arith, const bamf_batch_results *out, bamf_batch_graph **graph);
bamf_status bamf_rjmcmc_batch_graph_launch(bamf_batch_graph *graph, void *stream);
void bamf_rjmcmc_batch_graph_destroy(bamf_batch_graph *graph);

/* Autotuner (no reference counterpart): for every ROI size class present
 * in the (device) batch, times each CTA shape - 8, 4, 2 or 1 chains per CTA
 * in fast arithmetic, each with the kernel build whose registers are sized
 * for 2 or for 3 CTAs per SM, and (Gaussian PSF) one CTA of 24 chains per
 * SM, whose chains all follow one move stream; 4, 2 or 1 in exact - on the same ROIs of the
 * class for every shape (at least `sample` and at least three rounds of
 * the largest shape's resident chains, at most the class; evenly strided
 * through the class in the batch order, so that they span its whole photon
 * range) with chains of `jumps` burn-in jumps, and keeps the fastest shape
 * in the workspace; later bamf_rjmcmc_batch_device calls on that workspace launch
 * each class with its tuned shape.  Results of a batch do not depend on
 * the shape.  Synchronises `stream`. */
bamf_status bamf_autotune(bamf_workspace *ws, const bamf_roi_batch *rois, const bamf_mcmc_params *p,
                          const bamf_priors *priors, int arith, int jumps, int sample, void *stream);
/* chains_per_cta[7]: the tuned shape per size class (sides (0,8], (8,12],
 * ..., (28,32]); 0 where the class was not tuned. */
bamf_status bamf_autotune_result(const bamf_workspace *ws, int arith, int32_t *chains_per_cta);
/* The tuned shapes with the fast kernel's register budget: chains_per_cta
 * as bamf_autotune_result, ctas_per_sm_budget[c] the CTAs per SM the chosen
 * build's registers are sized for (fast: 1, 2 or 3; exact: 4; 0 untuned). */
bamf_status bamf_autotune_shapes(const bamf_workspace *ws, int arith, int32_t *chains_per_cta,
                                 int32_t *ctas_per_sm_budget);

/*
 * Allocation-free variant of bamf_rjmcmc_batch_device.  It has no
 * counterpart in the reference (which is a single-ROI CPU sampler).  It is
 * for callers that must not allocate device memory: hosts whose own pool
 * owns the device memory (MATLAB's gpuArray allocator, a framework's caching
 * allocator) and must not see the free memory change under them, and loops
 * that cannot take the device-wide synchronisation of cudaMalloc/cudaFree.
 * Same arguments and results as bamf_rjmcmc_batch_device minus the
 * workspace; it calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * Its scratch is one fixed array of BAMF_NOALLOC_SCRATCH_BYTES compiled into
 * the library: every GPU that loads the library holds it until the process
 * exits, and every call shares it.  A call needs
 *   512 + sum over the 3 priors of 16*len (each rounded up to 256)
 *   + 9*n_rois + 16 (the batch order; rounded up to 256)
 *   + [map_n wanted] n_rois*(N_Burnin+N_Trials) (+ 4*n_rois if n_entries is NULL)
 * bytes; a call needing more returns BAMF_ERR_TOO_LARGE before any GPU work
 * (split the batch).
 *
 * Set-up: the first call on each device looks up the array's device address
 * with that device current and keeps it for the life of the process.  The
 * address belongs to the device's context: after cudaDeviceReset of a
 * device, this entry point must not be called on that device again in the
 * same process.
 *
 * Priors: the three prior PDF arrays (priors->*_pdf) are host memory that
 * the call copies into the scratch with copies enqueued on `stream`.  From
 * ordinary (pageable) memory they are read before the call returns; from
 * page-locked memory (cudaHostAlloc / cudaHostRegister) the copies read them
 * when the stream reaches them, so such arrays must stay valid and unchanged
 * until then.
 *
 * Calls that overlap on the GPU (different streams, or different host
 * threads, not ordered by the caller) race on the shared scratch and
 * corrupt each other's results; calls on one stream are safe.  The
 * work-queue counters are cleared at the start of every call; nothing else
 * in the scratch is assumed to start at zero.  The size classes of a batch
 * run one after another on `stream` (the workspace entry point overlaps
 * them on side streams), so a batch of mixed ROI sizes takes somewhat longer.
 */
#define BAMF_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
bamf_status bamf_rjmcmc_batch_device_noalloc(const bamf_roi_batch *rois,
                                             const bamf_mcmc_params *p,
                                             const bamf_priors *priors, uint32_t seed,
                                             int arith, const bamf_batch_results *out,
                                             void *stream);

/* ------------------------------------------------------------------ */
/* Front end: findROI                                                   */
/* ------------------------------------------------------------------ */

/* Device scratch of the ROI finder (the DoG image and one byte of flags per
 * pixel of the stack, the filters' per-SM frame slots or, for frames of more
 * than about 80k pixels, a second image; chunk counts); grows on demand. */
typedef struct bamf_findroi_ws bamf_findroi_ws;
bamf_status bamf_findroi_workspace_create(bamf_findroi_ws **ws);
void bamf_findroi_workspace_destroy(bamf_findroi_ws *ws);

/*
 * findROI (@RJ/findROI.m:1-224 with the kernels of
 * source/cuda/cuda_FindROI/cuda_FindROI.cu): difference-of-Gaussians local
 * maxima of a frame stack.
 *   frames       ysize*xsize*zsize floats, y fastest (MATLAB Y x X x Z)
 *   sigma1/2     the two recursive-Gaussian widths (findROI.m Sigma1/Sigma2)
 *   boxsize      maximum-window half width and ROI side (Boxsize), at most
 *                128 (BAMF_ERR_TOO_LARGE beyond)
 *   minval       floor of the maxima (Minval), as the single the kernel gets
 *   capacity     rows available in coords/corners/roi_stack
 *   coords       [capacity][3] 1-based (row, col, frame) of each maximum in
 *                MATLAB find() order (findROI.m:125-126)
 *   corners      [capacity][2] (YBoxCorner, XBoxCorner) after the clamp of
 *                findROI.m:130-148, or NULL
 *   roi_stack    [capacity][boxsize*boxsize] crops, y fastest (findROI.m:157-160),
 *                or NULL (needs corners)
 *   count        number of maxima found (may exceed capacity: then only the
 *                first `capacity` are written)
 *   flags_out    optional ysize*xsize*zsize bytes, 1 at each maximum (Res)
 * _device: device pointers, count is a device int64, enqueued on stream.
 * _host: host pointers, synchronous.
 */
bamf_status bamf_find_roi_device(bamf_findroi_ws *ws, const float *frames, int ysize, int xsize,
                                 int zsize, double sigma1, double sigma2, int boxsize,
                                 float minval, int64_t capacity, int32_t *coords,
                                 int32_t *corners, float *roi_stack, int64_t *count,
                                 uint8_t *flags_out, void *stream);
bamf_status bamf_find_roi_host(const float *frames, int ysize, int xsize, int zsize,
                               double sigma1, double sigma2, int boxsize, float minval,
                               int64_t capacity, int32_t *coords, int32_t *corners,
                               float *roi_stack, int64_t *count);

/* bamf_find_roi_device on frames that are still in host memory: copies
 * host_frames (pinned, for the copies to overlap) into dev_frames (the
 * same size, device) in chunks of chunk_frames frames on a stream of the
 * workspace, and starts each chunk's row and column filters on `stream`
 * as soon as its copy has landed, then the window maxima of the chunk's
 * frames (those whose windows cannot reach a frame not yet filtered); the
 * compaction and crops run on the whole stack afterwards.  Outputs
 * identical to bamf_find_roi_device on the same frames.  Enqueued on stream;
 * host_frames must stay valid until the stream reaches this call's end. */
bamf_status bamf_find_roi_pinned(bamf_findroi_ws *ws, const float *host_frames, float *dev_frames,
                                 int chunk_frames, int ysize, int xsize, int zsize, double sigma1,
                                 double sigma2, int boxsize, float minval, int64_t capacity,
                                 int32_t *coords, int32_t *corners, float *roi_stack,
                                 int64_t *count, uint8_t *flags_out, void *stream);

/* bamf_find_roi_pinned followed by gaussMLE (XYNB, CCD; gaussMLE.m:92-205
 * with the ROI stack findROI.m:157-160 crops), chunk by chunk: after each
 * chunk's window maxima, the maxima of the flag chunks those complete are
 * appended to the coordinates in memory order, cropped and fitted while
 * later chunks are still being copied, so the work after the last copy is
 * the last chunk's.  coords, corners, roi_stack and count are
 * bamf_find_roi_pinned's (identical values); params and crlb are
 * [4][capacity]: bamf_gauss_mle_device's parameters (MATLAB Y, X, photons,
 * background) with the stride capacity, parameter k of ROI i at
 * k * capacity + i; loglik [capacity]; only the first min(count, capacity)
 * ROIs are written.
 * Device outputs, enqueued on stream; host_frames must stay valid until
 * the stream reaches this call's end.  boxsize up to 21 (the gaussMLE
 * window limit). */
bamf_status bamf_find_roi_fit_pinned(bamf_findroi_ws *ws, const float *host_frames, float *dev_frames,
                                     int chunk_frames, int ysize, int xsize, int zsize, double sigma1,
                                     double sigma2, int boxsize, float minval, int64_t capacity,
                                     float psf_sigma, int iterations, int32_t *coords,
                                     int32_t *corners, float *roi_stack, int64_t *count,
                                     float *params, float *crlb, float *loglik, void *stream);

/* The difference-of-Gaussians image findROI's maxima run on
 * (cuda_FindROI.cu kernel_gaussX / kernel_gaussY for sigma1 and sigma2, then
 * kernel_subtract): dog = G(sigma1) - G(sigma2) of each frame, in the frames'
 * layout (ysize*xsize*zsize floats, device).  Enqueued on stream. */
bamf_status bamf_find_roi_dog_device(bamf_findroi_ws *ws, const float *frames, int ysize, int xsize,
                                     int zsize, double sigma1, double sigma2, float *dog, void *stream);

/* The filters divide by the recurrence constant b0 with one multiply and
 * two FMAs through RN(1/b0) (Markstein's method) where |q| lies in
 * [2^-100, 2^100], after the host has checked, once per b0, that this equals
 * IEEE division over the 2^23 significands of [1, 2) (the method is
 * scale-invariant on that range); elsewhere, and for a b0 that fails the
 * check, they use IEEE division.  For the b0 of filter width `sigma`:
 * *host_exact = 1 when the host check passed.  With both counters given,
 * every one of the 2^32 float bit patterns q is also divided on the device
 * both ways: *dev_mismatch_in_range counts differing results with |q| in
 * the fast range (0 expected when *host_exact), *dev_mismatch all differing
 * results (NaN results compare equal).  Synchronous. */
bamf_status bamf_findroi_division_check(double sigma, int *host_exact,
                                        unsigned long long *dev_mismatch_in_range,
                                        unsigned long long *dev_mismatch);

/* ------------------------------------------------------------------ */
/* Front end: gaussMLE                                                  */
/* ------------------------------------------------------------------ */

/*
 * gaussMLE 'Basic' / 'CCD' (@RJ/gaussMLE.m:64-211, kernel_MLEFit_XYNB_ of
 * cuda_gaussMLEv2.cu:16-141): Newton-Raphson fit of (x, y, N, bg) per ROI.
 *   rois        nfits * sz * sz floats, each ROI y fastest (sz <= 21)
 *   iterations  Newton iterations (gaussMLE.m uses 20)
 *   params      [4][nfits] param-major: contiguous-axis position (MATLAB Y),
 *               other position (X), photons, background
 *   crlb        [4][nfits] Cramer-Rao lower bounds (variances)
 *   loglik      [nfits] log-likelihood ratio
 */
bamf_status bamf_gauss_mle_device(const float *rois, int sz, int nfits, float psf_sigma,
                                  int iterations, float *params, float *crlb, float *loglik,
                                  void *stream);
bamf_status bamf_gauss_mle_host(const float *rois, int sz, int nfits, float psf_sigma,
                                int iterations, float *params, float *crlb, float *loglik);

/* The other fit types of gaussMLE.m (FitType; cuda_gaussMLEv2.cu:144-1125):
 *   BAMF_FIT_BASIC    x, y, N, bg                    (NP 4, '_XYNB_')
 *   BAMF_FIT_SIGMA    + sigma                        (NP 5, '_XYNBS_')
 *   BAMF_FIT_Z        + z, astigmatic PSF (zfit)     (NP 5, '_XYNBZ_')
 *   BAMF_FIT_SIGMAYX  + sigma along each axis        (NP 6, '_XYNBSXSY_')
 * CameraType 'SCMOS' when var_gain_map is given: a map_size x map_size
 * variance / gain^2 image indexed at each ROI's box corner (box_corners
 * [n][2] floats: (axis-1 start, axis-0 start) as BoxCorners), '_SCMOS*_'.
 * Outputs param-major: params [NP][n], crlb [NP][n], loglik [n]; parameter
 * order (Y, X, Photons, BG, then Sigma | Z | SigmaY, SigmaX) as gaussMLE.m
 * unpacks them.  zfit: Sigma(1), Sigma(2) and ZStruct.Ax, Ay, Bx, By,
 * Gamma, D of gaussMLE.m:155-158. */
#define BAMF_FIT_BASIC 0
#define BAMF_FIT_SIGMA 1
#define BAMF_FIT_Z 2
#define BAMF_FIT_SIGMAYX 3
typedef struct bamf_zfit {
    float sigma_x, sigma_y;
    float Ax, Ay, Bx, By, gamma, d;
} bamf_zfit;
int bamf_gauss_mle_nparams(int fit_type);
bamf_status bamf_gauss_mle_fit_device(const float *rois, int sz, int nfits, int fit_type, float psf_sigma,
                                      const bamf_zfit *zfit, const float *box_corners, const float *var_gain_map,
                                      int map_size, int iterations, float *params, float *crlb, float *loglik,
                                      void *stream);
bamf_status bamf_gauss_mle_fit_host(const float *rois, int sz, int nfits, int fit_type, float psf_sigma,
                                    const bamf_zfit *zfit, const float *box_corners, const float *var_gain_map,
                                    int map_size, int iterations, float *params, float *crlb, float *loglik);

/* ------------------------------------------------------------------ */
/* Measurement helpers                                                  */
/* ------------------------------------------------------------------ */

/* Measured throughput of the two pipes the sampler runs on, on the
 * current device: dependent-free FP32 FMA (flop/s, 2 per FMA) and MUFU
 * log2 (op/s).  Runs two short probe kernels (~tens of ms); used as the
 * roofline denominators of the sampler.  Not used by any sampler path. */
bamf_status bamf_probe_peaks(double *fp32_flops, double *mufu_ops);

/* The erf (fn 0), log (1) and exp (2) of the exact sampler
 * (include/bamf_parity_math.h) evaluated on the device for n host inputs
 * x into host out: the same header compiled for the CPU must give the same
 * bits (the exact sampler's parity with the reference build rests on it).
 * Synchronous. */
bamf_status bamf_parity_math_device(int fn, const float *x, int n, float *out);

/* Known-answer check of the 5th-generation tensor-core path (tcgen05 MMA
 * from shared-memory descriptors into TMEM, read back with tcgen05.ld): a
 * 128 x 32 x 16 BF16 product of small integers.  *max_abs_err = the largest
 * deviation from the exact product (0 when the path works), *timed_out = 1
 * if the MMA's completion did not arrive within the kernel's bounded wait. */
bamf_status bamf_tcgen05_selftest(double *max_abs_err, int *timed_out);

/* The same check for one operand layout: 0 = both operands K-major (as
 * bamf_tcgen05_selftest), 1 = both MN-major (the layout of the
 * convolutions' weight-gradient GEMM). */
bamf_status bamf_tcgen05_selftest_layout(int layout, double *max_abs_err, int *timed_out);

#ifdef __cplusplus
}
#endif

#endif /* BAMF_H */
