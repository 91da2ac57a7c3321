/*
 * gaussmle.cu - single-emitter maximum-likelihood fits of (x, y, N, bg)
 * (gaussMLE 'Basic'/'CCD': kernel_MLEFit_XYNB_, cuda_gaussMLEv2.cu:16-141,
 * with GPUgaussLib.cuh:14-258 and MatInvLib.h:15-75) for sm_103a.
 *
 * A group of 8 lanes per fit (one thread per fit in the reference).  The model
 * is separable: the integrated PSF along x depends only on the column ii
 * and along y only on the row jj, and so do the x/y derivative factors up to
 * the final multiply by the other axis's PSF.  Those per-axis terms are
 * computed once per Newton iteration (2*sz values instead of sz^2), which
 * leaves every per-pixel value bit for bit what the direct evaluation gives.
 * The O(sz^4) start-up filter uses a table of the sz*2-1 distinct Gaussian
 * weights for the same reason.
 * Output layout as the reference: param-major P[Nfits*k + i], k = 0..3 for
 * (x along the contiguous axis, y, N, bg), CRLB likewise, LogLikelihood[i].
 */
#include <cuda_runtime.h>

#include "bamf.h"
#include "frontend_launch.h"

namespace {

constexpr int MAXSZ = GAUSS_MLE_MAX_SIZE; /* IMSZBIG of definitions.h: largest fit window */
#define MLE_PI 3.141592f         /* definitions.h:13 */

/* kernel_IntGauss1D (GPUgaussLib.cuh:14-24) */
__device__ __forceinline__ float int_gauss(int ii, float x, float sigma)
{
    const float norm = 1.0f / 2.0f / sigma / sigma;
    return 1.0f / 2.0f * (erff((ii - x + 1.0f) * sqrtf(norm)) - erff((ii - x) * sqrtf(norm)));
}

/* the part of kernel_DerivativeIntGauss1D (:67-87) before "* PSFother" */
__device__ __forceinline__ void dgauss_axis(int ii, float x, float sigma, float N, float *d1, float *d2)
{
    float u = (ii + 1.0f - x) / sigma, v = (ii - x) / sigma;
    float a = expf(-1.0f / 2.0f * (u * u));
    float b = expf(-1.0f / 2.0f * (v * v));
    *d1 = -N / sqrtf(2.0f * MLE_PI) / sigma * (a - b);
    *d2 = -N / sqrtf(2.0f * MLE_PI) / (sigma * sigma * sigma) * ((ii + 1.0f - x) * a - (ii - x) * b);
}

/* One fit per group of GL lanes (GL = 8: four fits per warp), ROIs staged
 * through shared memory with coalesced loads (the reference reads each ROI
 * per thread, uncoalesced).  Lane l of a group owns pixels l, l + GL, ...;
 * the centre of mass,
 * the start-up filter's positions, the Newton sums and the Fisher
 * information are lane partial sums (or maxima / minima) combined by
 * butterfly shuffles within the group, so every lane of the group holds
 * the same totals and the same theta.  The per-axis PSF and derivative
 * terms of an iteration are computed one value per lane into the group's
 * shared-memory rows.  The group's first lane inverts the 4 x 4 Fisher
 * matrix (MatInvLib.h:15-75) and writes the fit.  The reference's formulas
 * throughout; only the order of the pixel sums differs from its serial
 * loops. */
constexpr int GL = 8;
constexpr int GROUP_FITS_PER_BLOCK = 16; /* 128 threads */

__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = GL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* The nblk (<= GROUP_FITS_PER_BLOCK) fits from ROI `first` of `data`, by
 * the whole CTA; parameter k of fit i to P[stride * k + i] and CRLB alike,
 * the log-likelihood to LL[i].  Every thread returns here (lanes other than
 * a group's first return early). */
__device__ __forceinline__ void mle_xynb_block(const float *__restrict__ data, float sigma, int sz, int iterations,
                                               float *__restrict__ P, float *__restrict__ CRLB,
                                               float *__restrict__ LL, int64_t stride, int64_t first, int nblk)
{
    extern __shared__ float sm[];
    const int npx = sz * sz;
    /* coalesced staging of this block's ROIs; per fit 6 axis rows and the
     * start-up filter's weight table behind them */
    float *axis_all = sm + GROUP_FITS_PER_BLOCK * npx;
    /* pixel p -> (ii, jj) as ii << 8 | jj, once per block (no division in the
     * pixel loops) */
    int *pix = (int *)(axis_all + GROUP_FITS_PER_BLOCK * 8 * MAXSZ);
    for (int i = threadIdx.x; i < nblk * npx; i += blockDim.x) sm[i] = data[first * npx + i];
    for (int q = threadIdx.x; q < npx; q += blockDim.x) pix[q] = (q / sz) << 8 | (q % sz);
    __syncthreads();
    const int g = threadIdx.x / GL, l = threadIdx.x % GL;
    /* a group past the batch's end fits the block's first ROI again (its
     * lanes take part in the warp's shuffles) and writes nothing */
    const bool active = g < nblk;
    const float *d = sm + (active ? g : 0) * npx;
    float *px = axis_all + g * 6 * MAXSZ, *py = px + MAXSZ, *dx1 = py + MAXSZ, *dx2 = dx1 + MAXSZ,
          *dy1 = dx2 + MAXSZ, *dy2 = dy1 + MAXSZ;
    const int64_t fit = first + g;

    float theta[4];
    const float maxjump[4] = {1e0f, 1e0f, 1e2f, 2e0f};
    /* kernel_CenterofMass2D (GPUgaussLib.cuh:207-227) */
    float tx = 0.0f, ty = 0.0f, ts = 0.0f;
    for (int p = l; p < npx; p += GL) {
        const int ii = pix[p] >> 8, jj = pix[p] & 255; /* pixel d[sz*jj + ii] */
        const float v = d[sz * jj + ii];
        tx += v * ii;
        ty += v * jj;
        ts += v;
    }
    tx = group_sum(tx);
    ty = group_sum(ty);
    ts = group_sum(ts);
    theta[0] = tx / ts;
    theta[1] = ty / ts;
    /* kernel_GaussFMaxMin2D (:230-258): each lane filters its positions,
     * with the group's table of the 2 sz - 1 distinct Gaussian weights */
    float *w = axis_all + GROUP_FITS_PER_BLOCK * 6 * MAXSZ + g * (2 * MAXSZ);
    {
        const float norm = 1.0f / 2.0f / sigma / sigma;
        for (int q = l - (sz - 1); q <= sz - 1; q += GL) w[q + sz - 1] = expf(-(float)(q * q) * norm);
    }
    __syncwarp();
    float Nmax = 0.0f, MinBG = 10e10f;
    for (int pos = l; pos < npx; pos += GL) {
        const int kk = pix[pos] >> 8, ll = pix[pos] & 255;
        float fp = 0.0f, sum = 0.0f;
        for (int ii = 0; ii < sz; ii++)
            for (int jj = 0; jj < sz; jj++) {
                const float ww = w[ii - kk + sz - 1] * w[ll - jj + sz - 1];
                fp += ww * d[ii * sz + jj];
                sum += ww;
            }
        fp /= sum;
        Nmax = fmaxf(Nmax, fp);
        MinBG = fminf(MinBG, fp);
    }
#pragma unroll
    for (int o = GL / 2; o > 0; o >>= 1) {
        Nmax = fmaxf(Nmax, __shfl_xor_sync(0xffffffffu, Nmax, o));
        MinBG = fminf(MinBG, __shfl_xor_sync(0xffffffffu, MinBG, o));
    }
    theta[3] = MinBG;
    theta[2] = fmaxf(0.0f, (Nmax - theta[3]) * 2 * 2 * MLE_PI * sigma * sigma);

    for (int kk = 0; kk <= iterations; kk++) {
        /* the axis terms of theta (after the last iteration: for the Fisher
         * information) */
        for (int q = l; q < sz; q += GL) {
            px[q] = int_gauss(q, theta[0], sigma);
            py[q] = int_gauss(q, theta[1], sigma);
            dgauss_axis(q, theta[0], sigma, theta[2], &dx1[q], &dx2[q]);
            dgauss_axis(q, theta[1], sigma, theta[2], &dy1[q], &dy2[q]);
        }
        __syncwarp();
        if (kk == iterations) break;
        float num[4] = {0.0f, 0.0f, 0.0f, 0.0f}, den[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int p = l; p < npx; p += GL) {
            const int ii = pix[p] >> 8, jj = pix[p] & 255;
            const float PSFx = px[ii], PSFy = py[jj];
            const float model = theta[3] + theta[2] * PSFx * PSFy;
            const float data_v = d[sz * jj + ii];
            float dudt[4], d2udt2[4];
            dudt[0] = dx1[ii] * PSFy;
            d2udt2[0] = dx2[ii] * PSFy;
            dudt[1] = dy1[jj] * PSFx;
            d2udt2[1] = dy2[jj] * PSFx;
            dudt[2] = PSFx * PSFy;
            d2udt2[2] = 0.0f;
            dudt[3] = 1.0f;
            d2udt2[3] = 0.0f;
            float cf = 0.0f, df = 0.0f;
            if (model > 10e-3f) {
                const float r = __frcp_rn(model); /* data/model, data/model^2 as products */
                cf = data_v * r - 1;
                df = data_v * r * r;
            }
            cf = fminf(cf, 10e4f);
            df = fminf(df, 10e4f);
            for (int q = 0; q < 4; q++) {
                num[q] += dudt[q] * cf;
                den[q] += d2udt2[q] * cf - (dudt[q] * dudt[q]) * df;
            }
        }
        for (int q = 0; q < 4; q++) {
            num[q] = group_sum(num[q]);
            den[q] = group_sum(den[q]);
        }
        __syncwarp(); /* every lane has read the axis rows before they change */
        theta[0] -= fminf(fmaxf(num[0] / den[0], -maxjump[0]), maxjump[0]);
        theta[1] -= fminf(fmaxf(num[1] / den[1], -maxjump[1]), maxjump[1]);
        theta[2] -= fminf(fmaxf(num[2] / den[2], -theta[2]), theta[2]);
        theta[3] -= fminf(fmaxf(num[3] / den[3], -theta[3]), theta[3]);
        theta[2] = fmaxf(theta[2], 1.0f);
        theta[3] = fmaxf(theta[3], 0.01f);
    }

    /* Fisher information (10 distinct entries) and log-likelihood
     * (cuda_gaussMLEv2.cu:104-130) */
    float F[10] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float Div = 0.0f;
    for (int p = l; p < npx; p += GL) {
        const int ii = pix[p] >> 8, jj = pix[p] & 255;
        const float PSFx = px[ii], PSFy = py[jj];
        const float model = theta[3] + theta[2] * PSFx * PSFy;
        const float data_v = d[sz * jj + ii];
        const float dudt[4] = {dx1[ii] * PSFy, dy1[jj] * PSFx, PSFx * PSFy, 1.0f};
        const float rm = __frcp_rn(model);
        int e = 0;
        for (int a = 0; a < 4; a++)
            for (int b = a; b < 4; b++) F[e++] += dudt[b] * dudt[a] * rm;
        if (model > 0) {
            if (data_v > 0)
                Div += data_v * logf(model) - model - data_v * logf(data_v) + data_v;
            else
                Div += -model;
        }
    }
    for (int e = 0; e < 10; ++e) F[e] = group_sum(F[e]);
    Div = group_sum(Div);
    if (l != 0 || !active) return;
    float M[16];
    {
        int e = 0;
        for (int a = 0; a < 4; a++)
            for (int b = a; b < 4; b++) {
                M[a * 4 + b] = F[e];
                M[b * 4 + a] = F[e];
                ++e;
            }
    }
    /* kernel_MatInvN (MatInvLib.h:15-75): LU without pivoting, diagonal of
     * the inverse */
    const int n = 4;
    float Minv[16], yy[4], tmp1 = 0.0f;
    for (int jj = 0; jj < n; jj++) {
        for (int ii = 0; ii <= jj; ii++)
            if (ii > 0) {
                for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * n] * M[q + jj * n];
                M[ii + jj * n] -= tmp1;
                tmp1 = 0.0f;
            }
        for (int ii = jj + 1; ii < n; ii++)
            if (jj > 0) {
                for (int q = 0; q <= jj - 1; q++) tmp1 += M[ii + q * n] * M[q + jj * n];
                M[ii + jj * n] = (1 / M[jj + jj * n]) * (M[ii + jj * n] - tmp1);
                tmp1 = 0.0f;
            } else {
                M[ii + jj * n] = (1 / M[jj + jj * n]) * M[ii + jj * n];
            }
    }
    for (int num = 0; num < n; num++) {
        yy[0] = num == 0 ? 1.0f : 0.0f;
        for (int ii = 1; ii < n; ii++) {
            float b = ii == num ? 1.0f : 0.0f;
            for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * n] * yy[q];
            yy[ii] = b - tmp1;
            tmp1 = 0.0f;
        }
        Minv[n - 1 + num * n] = yy[n - 1] / M[(n - 1) + (n - 1) * n];
        for (int ii = n - 2; ii >= 0; ii--) {
            for (int q = ii + 1; q < n; q++) tmp1 += M[ii + q * n] * Minv[q + num * n];
            Minv[ii + num * n] = (1 / M[ii + ii * n]) * (yy[ii] - tmp1);
            tmp1 = 0.0f;
        }
    }
    for (int k = 0; k < 4; k++) {
        P[stride * k + fit] = theta[k];
        CRLB[stride * k + fit] = Minv[k * n + k];
    }
    LL[fit] = Div;
}

__global__ void __launch_bounds__(GL * GROUP_FITS_PER_BLOCK) mle_xynb_group_kernel(
    const float *__restrict__ data, float sigma, int sz, int iterations,
    float *__restrict__ P, float *__restrict__ CRLB, float *__restrict__ LL, int nfits)
{
    const int64_t first = (int64_t)blockIdx.x * GROUP_FITS_PER_BLOCK;
    mle_xynb_block(data, sigma, sz, iterations, P, CRLB, LL, nfits, first,
                   (int)min((int64_t)GROUP_FITS_PER_BLOCK, (int64_t)nfits - first));
}

/* The fits of ROIs [range[0], min(range[1], capacity)) of a stack whose
 * range is known only on the device: blocks of GROUP_FITS_PER_BLOCK fits,
 * grid-stride. */
__global__ void __launch_bounds__(GL * GROUP_FITS_PER_BLOCK) mle_xynb_range_kernel(
    const float *__restrict__ data, float sigma, int sz, int iterations, float *__restrict__ P,
    float *__restrict__ CRLB, float *__restrict__ LL, int64_t stride, const int64_t *__restrict__ range,
    int64_t capacity)
{
    const int64_t f0 = range[0], f1 = min(range[1], capacity);
    for (int64_t first = f0 + (int64_t)blockIdx.x * GROUP_FITS_PER_BLOCK; first < f1;
         first += (int64_t)gridDim.x * GROUP_FITS_PER_BLOCK) {
        mle_xynb_block(data, sigma, sz, iterations, P, CRLB, LL, stride, first,
                       (int)min((int64_t)GROUP_FITS_PER_BLOCK, f1 - first));
        __syncthreads(); /* the staged ROIs and axis rows are rewritten for the next fits */
    }
}

}  // namespace

static size_t gauss_mle_smem_bytes(int sz)
{
    return ((size_t)GROUP_FITS_PER_BLOCK * (sz * sz + 8 * MAXSZ) + (size_t)sz * sz) * sizeof(float);
}

bamf_status launch_gauss_mle_range(const float *rois, int sz, float psf_sigma, int iterations, float *params,
                                   float *crlb, float *loglik, int64_t stride, const int64_t *range,
                                   int64_t capacity, int blocks, cudaStream_t stream)
{
    if (sz < 1 || sz > MAXSZ || iterations < 0 || blocks < 1) return BAMF_ERR_INVALID_ARG;
    mle_xynb_range_kernel<<<blocks, GL * GROUP_FITS_PER_BLOCK, gauss_mle_smem_bytes(sz), stream>>>(
        rois, psf_sigma, sz, iterations, params, crlb, loglik, stride, range, capacity);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_gauss_mle_device(const float *rois, int sz, int nfits, float psf_sigma,
                                             int iterations, float *params, float *crlb,
                                             float *loglik, void *stream)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0 || iterations < 0)
        return BAMF_ERR_INVALID_ARG;
    if (sz > MAXSZ) return BAMF_ERR_TOO_LARGE;
    if (nfits == 0) return BAMF_OK;
    /* a group of GL lanes per fit: 16 fits per CTA of 128 threads */
    size_t smem = gauss_mle_smem_bytes(sz);
    int blocks = (nfits + GROUP_FITS_PER_BLOCK - 1) / GROUP_FITS_PER_BLOCK;
    mle_xynb_group_kernel<<<blocks, GL * GROUP_FITS_PER_BLOCK, smem, (cudaStream_t)stream>>>(
        rois, psf_sigma, sz, iterations, params, crlb, loglik, nfits);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_gauss_mle_host(const float *rois, int sz, int nfits, float psf_sigma,
                                           int iterations, float *params, float *crlb,
                                           float *loglik)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0 || iterations < 0)
        return BAMF_ERR_INVALID_ARG;
    if (sz > MAXSZ) return BAMF_ERR_TOO_LARGE;
    if (nfits == 0) return BAMF_OK;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    float *dr = nullptr, *dp = nullptr, *dc = nullptr, *dl = nullptr;
    size_t nin = (size_t)nfits * sz * sz, nout = (size_t)nfits * 4;
    bamf_status st = BAMF_OK;
    if (cudaMalloc(&dr, nin * sizeof(float)) != cudaSuccess || cudaMalloc(&dp, nout * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&dc, nout * sizeof(float)) != cudaSuccess || cudaMalloc(&dl, nfits * sizeof(float)) != cudaSuccess)
        st = BAMF_ERR_CUDA;
    if (!st && cudaMemcpy(dr, rois, nin * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st) st = bamf_gauss_mle_device(dr, sz, nfits, psf_sigma, iterations, dp, dc, dl, nullptr);
    if (!st && cudaDeviceSynchronize() != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st && (cudaMemcpy(params, dp, nout * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(crlb, dc, nout * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(loglik, dl, nfits * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess))
        st = BAMF_ERR_CUDA;
    cudaFree(dr);
    cudaFree(dp);
    cudaFree(dc);
    cudaFree(dl);
    return st;
}
