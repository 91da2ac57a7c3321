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
    cudaError_t e = cudaFuncSetAttribute(rjmcmc_kernel_sync<0>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    (void)K.sync_moves; /* always move-synchronous in fast arithmetic */
    rjmcmc_kernel_sync<0><<<blocks, 32 * warps_per_block, smem, stream>>>(K, B);
    return cudaGetLastError();
}

int blocks_per_sm_fast(int side_max, int warps_per_block)
{
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    if (cudaFuncSetAttribute(rjmcmc_kernel_sync<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rjmcmc_kernel_sync<0>, 32 * warps_per_block,
                                                      smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace bamf
