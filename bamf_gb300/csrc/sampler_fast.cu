/*
 * sampler_fast.cu - the fast sampler with the Gaussian PSF: hardware SFU
 * math, incremental model updates, warp-tree reductions, and
 * move-synchronous CTAs (the warps of a CTA draw the move type and jump
 * sub-branch from one shared stream and meet at a barrier before each jump,
 * so an SM's warps run the same code and the instruction cache stops
 * thrashing; each chain's move choice stays i.i.d. with the configured
 * probabilities and independent of its state).  Also the fast launchers,
 * which pick the likelihood model's build.
 */
#include "sampler_kernel.cuh"
#include "sampler_launch.h"

namespace bamf {

cudaError_t launch_fast_gauss(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                              int min_ctas, cudaStream_t stream)
{
    if (min_ctas == 1) return launch_kernel(rjmcmc_kernel_sync<false, 1>, K, B, smem, blocks, threads, stream);
    return min_ctas == 3 ? launch_kernel(rjmcmc_kernel_sync<false, 3>, K, B, smem, blocks, threads, stream)
                         : launch_kernel(rjmcmc_kernel_sync<false, 2>, K, B, smem, blocks, threads, stream);
}

int occupancy_fast_gauss(size_t smem, int threads, int min_ctas)
{
    if (min_ctas == 1) return resident_ctas(rjmcmc_kernel_sync<false, 1>, smem, threads);
    return min_ctas == 3 ? resident_ctas(rjmcmc_kernel_sync<false, 3>, smem, threads)
                         : resident_ctas(rjmcmc_kernel_sync<false, 2>, smem, threads);
}

cudaError_t launch_rjmcmc_fast(const SamplerConsts &K, const SamplerBatch &B, int side_max, int blocks,
                               int warps_per_block, int min_ctas, cudaStream_t stream)
{
    if (warps_per_block < 1 || BAMF_SYNC_GROUP % warps_per_block != 0) return cudaErrorInvalidValue;
    if (min_ctas < 1 || min_ctas > 3) return cudaErrorInvalidValue;
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    (void)K.sync_moves; /* always move-synchronous in fast arithmetic */
    return K.opt_model == 1 ? launch_fast_num(K, B, smem, blocks, 32 * warps_per_block, min_ctas, stream)
                            : launch_fast_gauss(K, B, smem, blocks, 32 * warps_per_block, min_ctas, stream);
}

int blocks_per_sm_fast(int side_max, int warps_per_block, int min_ctas, int opt_model)
{
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    return opt_model == 1 ? occupancy_fast_num(smem, 32 * warps_per_block, min_ctas)
                          : occupancy_fast_gauss(smem, 32 * warps_per_block, min_ctas);
}

int best_fast_shape(int side_max, int opt_model, int *warps_per_block, int *min_ctas)
{
    int best_w = 0, best_wpb = 8, best_mc = 2, best_per = 0;
    const int cand[3] = {8, 4, 2};
    for (int mc = 2; mc <= 3; ++mc)
        for (int i = 0; i < 3; ++i) {
            int per = blocks_per_sm_fast(side_max, cand[i], mc, opt_model);
            if (per * cand[i] > best_w) {
                best_w = per * cand[i];
                best_wpb = cand[i];
                best_mc = mc;
                best_per = per;
            }
        }
    /* up to side 12, one CTA of a whole move-stream group per SM (all of
     * the SM's warps on one instruction stream) measured faster than three
     * CTAs of 8 chains, when it keeps as many chains resident */
    if (side_max <= 12 && opt_model != 1) {
        const int per = blocks_per_sm_fast(side_max, BAMF_SYNC_GROUP, 1, opt_model);
        if (per * BAMF_SYNC_GROUP >= best_w) {
            best_wpb = BAMF_SYNC_GROUP;
            best_mc = 1;
            best_per = per;
        }
    }
    *warps_per_block = best_wpb;
    *min_ctas = best_mc;
    return best_per;
}

}  // namespace bamf
