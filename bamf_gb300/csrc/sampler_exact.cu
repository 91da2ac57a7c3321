/*
 * sampler_exact.cu - the exact (parity) instantiation of the sampler kernel.
 * Built with -fmad=false so that no float multiply-add is fused: every
 * operation rounds as in the reference's x86 SSE build.
 */
#include "sampler_kernel.cuh"

namespace bamf {

cudaError_t launch_rjmcmc_exact(const SamplerConsts &K, const SamplerBatch &B, int side_max,
                                int blocks, int warps_per_block, cudaStream_t stream)
{
    size_t smem = (size_t)warp_smem_floats(side_max, true) * sizeof(float) * warps_per_block;
    auto kern = K.opt_model == 1 ? rjmcmc_kernel<true, true> : rjmcmc_kernel<true, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<blocks, 32 * warps_per_block, smem, stream>>>(K, B);
    return cudaGetLastError();
}

int blocks_per_sm_exact(int side_max, int warps_per_block, int opt_model)
{
    size_t smem = (size_t)warp_smem_floats(side_max, true) * sizeof(float) * warps_per_block;
    auto kern = opt_model == 1 ? rjmcmc_kernel<true, true> : rjmcmc_kernel<true, false>;
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
