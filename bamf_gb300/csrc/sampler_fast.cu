/*
 * sampler_fast.cu - the fast instantiation of the sampler kernel: hardware
 * SFU math, incremental model updates, warp-tree reductions.
 */
#include "sampler_kernel.cuh"

namespace bamf {

cudaError_t launch_rjmcmc_fast(const SamplerConsts &K, const SamplerBatch &B, int side_max,
                               int blocks, int warps_per_block, cudaStream_t stream)
{
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    cudaError_t e = cudaFuncSetAttribute(rjmcmc_kernel<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    rjmcmc_kernel<false><<<blocks, 32 * warps_per_block, smem, stream>>>(K, B);
    return cudaGetLastError();
}

int blocks_per_sm_fast(int side_max, int warps_per_block)
{
    size_t smem = (size_t)warp_smem_floats(side_max, false) * sizeof(float) * warps_per_block;
    if (cudaFuncSetAttribute(rjmcmc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rjmcmc_kernel<false>, 32 * warps_per_block,
                                                      smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace bamf
