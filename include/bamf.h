/*
 * bamf.h - C ABI of the GB300-native BAMF hot path (libbamf_gb300.so).
 *
 * Three groups of entry points, each replacing one reference interface:
 *   - the reversible-jump sampler   (MEX cRJMCMC, source/c/cRJMCMC.cpp:52-308)
 *   - the ROI finder                (findROI, @RJ/findROI.m:1-224 driving
 *                                    source/cuda/cuda_FindROI/cuda_FindROI.cu)
 *   - the single-emitter MLE fitter (gaussMLE, @RJ/gaussMLE.m:64-211 driving
 *                                    kernel_MLEFit_XYNB_, cuda_gaussMLEv2.cu:16-141)
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

#ifdef __cplusplus
}
#endif

#endif /* BAMF_H */
