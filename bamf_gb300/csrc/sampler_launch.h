/*
 * sampler_launch.h - launchers of the sampler kernels, one translation unit
 * per (arithmetic, likelihood model) so the four builds compile in
 * parallel.  The fast kernel exists in two register budgets: for 2 CTAs of
 * 8 chains per SM (no spills) and for 3 (80 registers, a few spills), which
 * keeps a third CTA resident where shared memory allows (ROI sides <= 20).
 */
#ifndef BAMF_SAMPLER_LAUNCH_H
#define BAMF_SAMPLER_LAUNCH_H

#include <cuda_runtime.h>

#include "sampler_common.h"

namespace bamf {

/* fast arithmetic: min_ctas = the kernel's register budget (2 or 3 CTAs per SM) */
cudaError_t launch_rjmcmc_fast(const SamplerConsts &K, const SamplerBatch &B, int side_max, int blocks,
                               int warps_per_block, int min_ctas, cudaStream_t stream);
int blocks_per_sm_fast(int side_max, int warps_per_block, int min_ctas, int opt_model);
cudaError_t launch_rjmcmc_exact(const SamplerConsts &K, const SamplerBatch &B, int side_max, int blocks,
                                int warps_per_block, cudaStream_t stream);
int blocks_per_sm_exact(int side_max, int warps_per_block, int opt_model);

/* the CTA shape with the most resident chains per SM for a fast launch
 * (ties: the larger register budget per thread, then more chains per CTA;
 * up to side 12, a whole move-stream group per CTA when it keeps as many) */
int best_fast_shape(int side_max, int opt_model, int *warps_per_block, int *min_ctas);

/* per translation unit */
cudaError_t launch_fast_gauss(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                              int min_ctas, cudaStream_t stream);
int occupancy_fast_gauss(size_t smem, int threads, int min_ctas);
cudaError_t launch_fast_num(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                            int min_ctas, cudaStream_t stream);
int occupancy_fast_num(size_t smem, int threads, int min_ctas);
cudaError_t launch_exact_gauss(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                               cudaStream_t stream);
int occupancy_exact_gauss(size_t smem, int threads);
cudaError_t launch_exact_num(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                             cudaStream_t stream);
int occupancy_exact_num(size_t smem, int threads);

/* set the kernel's dynamic shared memory and launch it */
template <typename Kern>
inline cudaError_t launch_kernel(Kern kern, const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks,
                                 int threads, cudaStream_t stream)
{
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<blocks, threads, smem, stream>>>(K, B);
    return cudaGetLastError();
}

/* resident CTAs per SM of the kernel at this shape; 0 when it does not fit */
template <typename Kern>
inline int resident_ctas(Kern kern, size_t smem, int threads)
{
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace bamf

#endif
