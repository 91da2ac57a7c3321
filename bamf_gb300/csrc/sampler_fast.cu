/*
 * sampler_fast.cu - the fast sampler: hardware SFU math, incremental model
 * updates, warp-tree reductions, and move-synchronous CTAs (the warps of a
 * CTA draw the move type and jump sub-branch from one shared stream and meet
 * at a barrier before each jump, so an SM's warps run the same code and the
 * instruction cache stops thrashing; each chain's move choice stays i.i.d.
 * with the configured probabilities and independent of its state).
 */
#include "sampler_kernel.cuh"

namespace bamf {

cudaError_t launch_rjmcmc_fast(const SamplerConsts &K, const SamplerBatch &B, int side_max,
                               int blocks, int warps_per_block, cudaStream_t stream)
{
    if (warps_per_block < 1 || BAMF_SYNC_GROUP % warps_per_block != 0) return cudaErrorInvalidValue;
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    /* one instantiation per likelihood model, so the Gaussian path carries
     * no sampled-PSF code */
    auto kern = K.opt_model == 1 ? rjmcmc_kernel_sync<true> : rjmcmc_kernel_sync<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    (void)K.sync_moves; /* always move-synchronous in fast arithmetic */
    kern<<<blocks, 32 * warps_per_block, smem, stream>>>(K, B);
    return cudaGetLastError();
}

int blocks_per_sm_fast(int side_max, int warps_per_block, int opt_model)
{
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    auto kern = opt_model == 1 ? rjmcmc_kernel_sync<true> : rjmcmc_kernel_sync<false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, 32 * warps_per_block, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace bamf
