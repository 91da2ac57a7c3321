/*
 * mapfit.cu - the chain summaries that follow the sampler in the reference's
 * analysis, on the device, from the thinned state records of the batched
 * sampler (bamf_batch_results.pos_trace):
 *
 *   findMap.m:29-111  MAP emitter count over the second half of the chain,
 *                     k-means (k = MAP count) of the positions of the states
 *                     with that count, and per-cluster mean / standard
 *                     deviation of X, Y, I; mean / std of the background
 *   mcmc.m:142-169    per-emitter mean / standard deviation over the second
 *                     half of a fixed-count (jumps-only) chain
 *
 * "Second half" is the reference's: with L = chain entries - 1 (the MEX
 * output drops the last entry), entries round(L/2) .. L (1-based) of the
 * accepted chain, i.e. 0-based entries ceil(L/2)-1 .. L-1, restricted here
 * to the recorded ones (every pos_thin-th entry).
 *
 * k-means: Lloyd iterations with squared Euclidean distance (ties to the
 * lower cluster), started from the emitters of the first qualifying state
 * (distinct points of one posterior sample), until no assignment changes
 * or max_iter; an empty cluster keeps its centre.  MATLAB's kmeans starts
 * from random k-means++ seeds, so cluster order and the last digits differ;
 * the clusters themselves are the same partition of a well-separated
 * posterior.  Standard deviations use n - 1 (MATLAB std); one point gives 0.
 */
#include <cuda_runtime.h>

#include <cmath>

#include "bamf.h"

/* a failed CUDA runtime call: clear its error so that a later call on this
 * thread does not report it again */
static inline bamf_status clear_cuda_error()
{
    cudaGetLastError();
    return BAMF_ERR_CUDA;
}

namespace {

constexpr int S = BAMF_POS_SLOTS;
constexpr int REC = BAMF_POS_RECORD;
constexpr int THREADS = 128;
constexpr int MAX_POS_LEN = 256;

__device__ __forceinline__ float nanf_() { return __int_as_float(0x7fc00000); }

/* block sum of a double (deterministic tree) */
__device__ double block_sum(double v, double *red)
{
    const int t = threadIdx.x;
    red[t] = v;
    __syncthreads();
    for (int o = THREADS / 2; o > 0; o >>= 1) {
        if (t < o) red[t] += red[t + o];
        __syncthreads();
    }
    double r = red[0];
    __syncthreads();
    return r;
}

struct Range {
    int lo, hi; /* qualifying 0-based entries lo .. hi */
};

__device__ __forceinline__ Range second_half(int n_entries)
{
    int iter = n_entries - 1;
    Range r;
    r.lo = (iter + 1) / 2 - 1;
    r.hi = iter - 1;
    return r;
}

__global__ void __launch_bounds__(THREADS) map_kmeans_kernel(const float *__restrict__ pos, int pos_len,
                                                             int pos_thin, const int32_t *__restrict__ n_entries,
                                                             const int32_t *__restrict__ map_n, int n,
                                                             int max_iter, float *__restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *PX = (float *)smem_raw;
    float *PY = PX + MAX_POS_LEN * S;
    float *PI = PY + MAX_POS_LEN * S;
    int *asg = (int *)(PI + MAX_POS_LEN * S);
    __shared__ double red[THREADS];
    __shared__ int qpos[THREADS + 1];
    __shared__ float cx[S], cy[S];
    __shared__ int changed, npts_sh;
    const int roi = blockIdx.x, t = threadIdx.x;
    if (roi >= n) return;
    float *o = out + (int64_t)roi * BAMF_MAP_RECORD;
    const float *rp = pos + (int64_t)roi * pos_len * REC;
    const Range rg = second_half(n_entries[roi]);
    const int nw = min(pos_len, (n_entries[roi] + pos_thin - 1) / pos_thin); /* records written */
    const int K = min(max(map_n[roi], 0), S);
    /* gather qualifying records in record order */
    if (t == 0) npts_sh = 0;
    __syncthreads();
    double sb = 0.0, sb2 = 0.0, sa = 0.0, sbb = 0.0, cnt = 0.0;
    for (int b0 = 0; b0 < nw; b0 += THREADS) {
        int r = b0 + t;
        bool q = false;
        const float *rec = rp + (int64_t)min(r, nw - 1) * REC;
        if (r < nw) {
            int e = r * pos_thin;
            q = rec[1] == (float)K && e >= rg.lo && e <= rg.hi;
        }
        if (q) {
            sb += rec[2];
            sb2 += (double)rec[2] * rec[2];
            sa += rec[3];
            sbb += rec[4];
            cnt += 1.0;
        }
        /* exclusive scan of q over the block */
        qpos[t] = q ? 1 : 0;
        __syncthreads();
        if (t == 0) {
            int acc = npts_sh;
            for (int k = 0; k < THREADS; ++k) {
                int v = qpos[k];
                qpos[k] = acc;
                acc += v;
            }
            qpos[THREADS] = acc;
        }
        __syncthreads();
        if (q && K > 0)
            for (int s = 0; s < K; ++s) {
                int p = qpos[t] * K + s;
                PX[p] = rec[5 + s];
                PY[p] = rec[5 + S + s];
                PI[p] = rec[5 + 2 * S + s];
            }
        __syncthreads();
        if (t == 0) npts_sh = qpos[THREADS];
        __syncthreads();
    }
    const int nrec = npts_sh, npts = nrec * K;
    double tb = block_sum(sb, red), tb2 = block_sum(sb2, red), ta = block_sum(sa, red);
    double tbb = block_sum(sbb, red), tc = block_sum(cnt, red);
    if (t == 0) {
        o[0] = (float)K;
        o[1] = (float)nrec;
        o[2] = tc > 0 ? (float)(tb / tc) : nanf_();
        o[3] = tc > 1 ? (float)sqrt(fmax(0.0, (tb2 - tb * tb / tc) / (tc - 1.0))) : (tc == 1 ? 0.0f : nanf_());
        o[4] = tc > 0 ? (float)(ta / tc) : nanf_();
        o[5] = tc > 0 ? (float)(tbb / tc) : nanf_();
    }
    for (int s = t; s < 6 * S; s += THREADS) o[6 + s] = nanf_();
    __syncthreads();
    if (K == 0 || nrec == 0) return;
    /* Lloyd iterations */
    if (t < K) {
        cx[t] = PX[t];
        cy[t] = PY[t];
    }
    for (int p = t; p < npts; p += THREADS) asg[p] = -1;
    __syncthreads();
    for (int it = 0; it < max_iter; ++it) {
        if (t == 0) changed = 0;
        __syncthreads();
        for (int p = t; p < npts; p += THREADS) {
            float bx = PX[p], by = PY[p];
            int best = 0;
            float bd = INFINITY;
            for (int c = 0; c < K; ++c) {
                float dx = bx - cx[c], dy = by - cy[c];
                float d = dx * dx + dy * dy;
                if (d < bd) {
                    bd = d;
                    best = c;
                }
            }
            if (asg[p] != best) {
                asg[p] = best;
                changed = 1;
            }
        }
        __syncthreads();
        if (!changed) break;
        for (int c = 0; c < K; ++c) {
            double sx = 0.0, sy = 0.0, sn = 0.0;
            for (int p = t; p < npts; p += THREADS)
                if (asg[p] == c) {
                    sx += PX[p];
                    sy += PY[p];
                    sn += 1.0;
                }
            double SX = block_sum(sx, red), SY = block_sum(sy, red), SN = block_sum(sn, red);
            if (t == 0 && SN > 0) {
                cx[c] = (float)(SX / SN);
                cy[c] = (float)(SY / SN);
            }
            __syncthreads();
        }
    }
    /* per-cluster mean and standard deviation of X, Y, I */
    for (int c = 0; c < K; ++c) {
        double a[3] = {0, 0, 0}, a2[3] = {0, 0, 0}, sn = 0;
        for (int p = t; p < npts; p += THREADS)
            if (asg[p] == c) {
                double v[3] = {PX[p], PY[p], PI[p]};
                for (int k = 0; k < 3; ++k) {
                    a[k] += v[k];
                    a2[k] += v[k] * v[k];
                }
                sn += 1.0;
            }
        double N = block_sum(sn, red);
        for (int k = 0; k < 3; ++k) {
            double A = block_sum(a[k], red), A2 = block_sum(a2[k], red);
            if (t == 0) {
                o[6 + k * S + c] = N > 0 ? (float)(A / N) : nanf_();
                o[6 + (3 + k) * S + c] =
                    N > 1 ? (float)sqrt(fmax(0.0, (A2 - A * A / N) / (N - 1.0))) : (N == 1 ? 0.0f : nanf_());
            }
        }
    }
}

/* mcmc.m:142-169: per-slot mean and std over the second half of a
 * fixed-count chain (the count is taken from the first record in range) */
__global__ void __launch_bounds__(THREADS) refine_stats_kernel(const float *__restrict__ pos, int pos_len,
                                                               int pos_thin, const int32_t *__restrict__ n_entries,
                                                               int n, float *__restrict__ out)
{
    __shared__ double red[THREADS];
    const int roi = blockIdx.x, t = threadIdx.x;
    if (roi >= n) return;
    float *o = out + (int64_t)roi * BAMF_MAP_RECORD;
    const float *rp = pos + (int64_t)roi * pos_len * REC;
    const Range rg = second_half(n_entries[roi]);
    const int nw = min(pos_len, (n_entries[roi] + pos_thin - 1) / pos_thin);
    /* records r in range: rg.lo <= r * pos_thin <= rg.hi */
    const int r0 = max(0, (rg.lo + pos_thin - 1) / pos_thin);
    const int r1 = min(nw - 1, rg.hi >= 0 ? rg.hi / pos_thin : -1);
    const int nrec = max(0, r1 - r0 + 1);
    const int kf = nrec > 0 ? min((int)rp[(int64_t)r0 * REC + 1], S) : 0;
    const double tn = (double)nrec;
    if (t == 0) {
        o[0] = (float)kf;
        o[1] = (float)nrec;
        o[2] = o[3] = o[4] = o[5] = nanf_();
    }
    for (int s = t; s < 6 * S; s += THREADS) o[6 + s] = nanf_();
    __syncthreads();
    for (int s = 0; s < kf; ++s)
        for (int k = 0; k < 3; ++k) {
            double a = 0.0, a2 = 0.0;
            for (int r = r0 + t; r <= r1; r += THREADS) {
                double v = rp[(int64_t)r * REC + 5 + k * S + s];
                a += v;
                a2 += v * v;
            }
            double A = block_sum(a, red), A2 = block_sum(a2, red);
            if (t == 0) {
                o[6 + k * S + s] = tn > 0 ? (float)(A / tn) : nanf_();
                o[6 + (3 + k) * S + s] =
                    tn > 1 ? (float)sqrt(fmax(0.0, (A2 - A * A / tn) / (tn - 1.0))) : (tn == 1 ? 0.0f : nanf_());
            }
        }
}

}  // namespace

extern "C" bamf_status bamf_map_kmeans_device(const float *pos_trace, int pos_len, int pos_thin,
                                              const int32_t *n_entries, const int32_t *map_n, int n, int max_iter,
                                              float *out, void *stream)
{
    if (n < 0 || pos_len < 1 || pos_len > MAX_POS_LEN || pos_thin < 1 || max_iter < 1) return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    if (!pos_trace || !n_entries || !map_n || !out) return BAMF_ERR_INVALID_ARG;
    size_t smem = (size_t)MAX_POS_LEN * S * (3 * sizeof(float) + sizeof(int));
    if (cudaFuncSetAttribute(map_kmeans_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return clear_cuda_error();
    map_kmeans_kernel<<<n, THREADS, smem, (cudaStream_t)stream>>>(pos_trace, pos_len, pos_thin, n_entries, map_n,
                                                                  n, max_iter, out);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_refine_stats_device(const float *pos_trace, int pos_len, int pos_thin,
                                                const int32_t *n_entries, int n, float *out, void *stream)
{
    if (n < 0 || pos_len < 1 || pos_thin < 1) return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    if (!pos_trace || !n_entries || !out) return BAMF_ERR_INVALID_ARG;
    refine_stats_kernel<<<n, THREADS, 0, (cudaStream_t)stream>>>(pos_trace, pos_len, pos_thin, n_entries, n, out);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}
