/*
 * sampler_exact.cu - the exact (parity) sampler with the Gaussian PSF, and
 * the exact launchers.  Built with -fmad=false so that no float
 * multiply-add is fused: every operation rounds as in the reference's x86
 * SSE build.
 */
#include "sampler_kernel.cuh"
#include "sampler_launch.h"

namespace bamf {

cudaError_t launch_exact_gauss(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                               cudaStream_t stream)
{
    return launch_kernel(rjmcmc_kernel<true, false>, K, B, smem, blocks, threads, stream);
}

int occupancy_exact_gauss(size_t smem, int threads) { return resident_ctas(rjmcmc_kernel<true, false>, smem, threads); }

cudaError_t launch_rjmcmc_exact(const SamplerConsts &K, const SamplerBatch &B, int side_max, int blocks,
                                int warps_per_block, cudaStream_t stream)
{
    size_t smem = (size_t)warp_smem_floats(side_max, true) * sizeof(float) * warps_per_block;
    return K.opt_model == 1 ? launch_exact_num(K, B, smem, blocks, 32 * warps_per_block, stream)
                            : launch_exact_gauss(K, B, smem, blocks, 32 * warps_per_block, stream);
}

int blocks_per_sm_exact(int side_max, int warps_per_block, int opt_model)
{
    size_t smem = (size_t)warp_smem_floats(side_max, true) * sizeof(float) * warps_per_block;
    return opt_model == 1 ? occupancy_exact_num(smem, 32 * warps_per_block)
                          : occupancy_exact_gauss(smem, 32 * warps_per_block);
}

}  // namespace bamf
