/*
 * gaussmle_fits.cu - the other gaussMLE fit types (@RJ/gaussMLE.m FitType
 * 'Sigma', 'Z', 'SigmaYX', and CameraType 'SCMOS' for all four types) with
 * the reference kernels' Newton-Raphson updates, constraints, Fisher
 * information and log-likelihood (cuda_gaussMLEv2.cu:144-1125 with
 * GPUgaussLib.cuh:14-258 and MatInvLib.h:15-75).  CCD 'Basic' has its own
 * optimised kernel (gaussmle.cu).
 *
 * One group of 8 lanes per fit (four fits per warp), the block's ROIs staged
 * through shared memory with coalesced loads; lane l of a group evaluates
 * pixels l, l + 8, ..., and the group's partial sums (centre of mass,
 * Newton numerators and denominators, Fisher information, log-likelihood)
 * and the start-up filter's maximum and minimum are combined by butterfly
 * shuffles, so all lanes of a group carry the same parameters.  Parameters
 * theta: 0 = position along the contiguous
 * ROI axis (MATLAB rows: Results.Y), 1 = the other axis (Results.X),
 * 2 = photons, 3 = background, then
 *   Sigma:   4 = sigma of a symmetric PSF
 *   Z:       4 = z of an astigmatic PSF, sigma_a = sigma_a0 sqrt(alpha_a(z)),
 *            alpha_a(z) = 1 + (z'/d)^2 + A_a (z'/d)^3 + B_a (z'/d)^4 with
 *            z' = z - gamma along axis 0 and z + gamma along axis 1
 *   SigmaYX: 4, 5 = sigma along axis 0 and axis 1
 * sCMOS: every pixel's variance-to-gain ratio g (from a square map, at the
 * ROI's box corner) enters as cf = (data - model)/(model + g),
 * df = (data + g)/(model + g)^2.  The reference's CRLB / log-likelihood pass
 * does not re-read g per pixel: it uses the value left from the last pixel
 * of the last Newton iteration, (sz-1, sz-1), and so does this code (0 when
 * there are no iterations, where the reference reads an uninitialised
 * value).
 */
#include <cuda_runtime.h>

#include "bamf.h"

namespace {

constexpr int MAXSZ = 21;
constexpr int FITS_PER_BLOCK = 16; /* fits per CTA, 8 lanes each */
#define MLE_PI 3.141592f

struct ZPar {
    float sx, sy, Ax, Ay, Bx, By, gamma, d;
};

__device__ __forceinline__ float int_gauss(int ii, float x, float sigma)
{
    const float norm = 1.0f / 2.0f / sigma / sigma;
    return 1.0f / 2.0f * (erff((ii - x + 1.0f) * sqrtf(norm)) - erff((ii - x) * sqrtf(norm)));
}

/* kernel_DerivativeIntGauss1D (GPUgaussLib.cuh:67-87) */
__device__ __forceinline__ void d_gauss(int ii, float x, float sigma, float N, float other, float *d1, float *d2)
{
    float a = expf(-1.0f / 2.0f * ((ii + 1.0f - x) / sigma) * ((ii + 1.0f - x) / sigma));
    float b = expf(-1.0f / 2.0f * ((ii - x) / sigma) * ((ii - x) / sigma));
    *d1 = -N / sqrtf(2.0f * MLE_PI) / sigma * (a - b) * other;
    if (d2) *d2 = -N / sqrtf(2.0f * MLE_PI) / (sigma * sigma * sigma) * ((ii + 1.0f - x) * a - (ii - x) * b) * other;
}

/* kernel_DerivativeIntGauss1DSigma (:90-110) */
__device__ __forceinline__ void d_gauss_sigma(int ii, float x, float S, float N, float other, float *d1, float *d2)
{
    float u = ii - x + 1.0f, v = ii - x;
    float a = expf(-1.0f / 2.0f * (u / S) * (u / S));
    float b = expf(-1.0f / 2.0f * (v / S) * (v / S));
    float g = -N / sqrtf(2.0f * MLE_PI) / S / S * (a * u - b * v) * other;
    *d1 = g;
    if (d2) {
        float S5 = S * S * S * S * S;
        *d2 = -2.0f / S * g - N / sqrtf(2.0f * MLE_PI) / S5 * (a * u * u * u - b * v * v * v) * other;
    }
}

/* kernel_alpha and its z-derivatives (:25-57) */
__device__ __forceinline__ float alpha_z(float z, float A, float B, float d)
{
    float t = z / d;
    return 1.0f + t * t + A * t * t * t + B * t * t * t * t;
}
__device__ __forceinline__ float dalpha_z(float z, float A, float B, float d)
{
    return 2.0f * z / (d * d) + 3.0f * A * z * z / (d * d * d) + 4.0f * B * z * z * z / (d * d * d * d);
}
__device__ __forceinline__ float d2alpha_z(float z, float A, float B, float d)
{
    return 2.0f / (d * d) + 6.0f * A * z / (d * d * d) + 12.0f * B * z * z / (d * d * d * d);
}

/* model terms of pixel (ii, jj): PSF along both axes, dudt, d2udt2 */
template <int FIT>
__device__ __forceinline__ void pixel(int ii, int jj, const float *th, float sigma, const ZPar &z, float *px,
                                      float *py, float *du, float *d2u)
{
    if (FIT == BAMF_FIT_BASIC || FIT == BAMF_FIT_SIGMA || FIT == BAMF_FIT_SIGMAYX) {
        float s0 = FIT == BAMF_FIT_BASIC ? sigma : th[4];
        float s1 = FIT == BAMF_FIT_SIGMAYX ? th[5] : s0;
        float PSFx = int_gauss(ii, th[0], s0), PSFy = int_gauss(jj, th[1], s1);
        d_gauss(ii, th[0], s0, th[2], PSFy, &du[0], d2u ? &d2u[0] : nullptr);
        d_gauss(jj, th[1], s1, th[2], PSFx, &du[1], d2u ? &d2u[1] : nullptr);
        if (FIT == BAMF_FIT_SIGMA) {
            float a, b, c, e;
            d_gauss_sigma(ii, th[0], s0, th[2], PSFy, &a, &b);
            d_gauss_sigma(jj, th[1], s0, th[2], PSFx, &c, &e);
            du[4] = a + c;
            if (d2u) d2u[4] = b + e;
        }
        if (FIT == BAMF_FIT_SIGMAYX) {
            d_gauss_sigma(ii, th[0], s0, th[2], PSFy, &du[4], d2u ? &d2u[4] : nullptr);
            d_gauss_sigma(jj, th[1], s1, th[2], PSFx, &du[5], d2u ? &d2u[5] : nullptr);
        }
        *px = PSFx;
        *py = PSFy;
    } else { /* Z: kernel_DerivativeIntGauss2Dz (:135-205) */
        float zz = th[4];
        float ax = alpha_z(zz - z.gamma, z.Ax, z.Bx, z.d), ay = alpha_z(zz + z.gamma, z.Ay, z.By, z.d);
        float Sx = z.sx * sqrtf(ax), Sy = z.sy * sqrtf(ay);
        float PSFx = int_gauss(ii, th[0], Sx), PSFy = int_gauss(jj, th[1], Sy);
        float ddx, ddy, dSx, dSy, ddSx, ddSy;
        d_gauss(ii, th[0], Sx, th[2], PSFy, &du[0], &ddx);
        d_gauss(jj, th[1], Sy, th[2], PSFx, &du[1], &ddy);
        d_gauss_sigma(ii, th[0], Sx, th[2], PSFy, &dSx, &ddSx);
        d_gauss_sigma(jj, th[1], Sy, th[2], PSFx, &dSy, &ddSy);
        float dSax = z.sx / 2.0f / sqrtf(ax), dSay = z.sy / 2.0f / sqrtf(ay);
        float dzx = dalpha_z(zz - z.gamma, z.Ax, z.Bx, z.d), dzy = dalpha_z(zz + z.gamma, z.Ay, z.By, z.d);
        float dSdzx = dSax * dzx, dSdzy = dSay * dzy;
        du[4] = dSx * dSdzx + dSy * dSdzy;
        if (d2u) {
            d2u[0] = ddx;
            d2u[1] = ddy;
            float d2Sax = -z.sx / 4.0f / (ax * sqrtf(ax)), d2Say = -z.sy / 4.0f / (ay * sqrtf(ay));
            float ddSddzx = d2Sax * dzx * dzx + dSax * d2alpha_z(zz - z.gamma, z.Ax, z.Bx, z.d);
            float ddSddzy = d2Say * dzy * dzy + dSay * d2alpha_z(zz + z.gamma, z.Ay, z.By, z.d);
            d2u[4] = ddSx * (dSdzx * dSdzx) + dSx * ddSddzx + ddSy * (dSdzy * dSdzy) + dSy * ddSddzy;
        }
        *px = PSFx;
        *py = PSFy;
    }
    du[2] = *px * *py;
    du[3] = 1.0f;
    if (d2u) {
        d2u[2] = 0.0f;
        d2u[3] = 0.0f;
    }
}

constexpr int GL = 8; /* lanes per fit: four fits per warp */

__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = GL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int FIT, bool SCMOS>
__global__ void __launch_bounds__(GL * FITS_PER_BLOCK) mle_fit_kernel(
    const float *__restrict__ data, float sigma, ZPar zp, const float *__restrict__ coords,
    const float *__restrict__ gmap, int mapsz, int sz, int iterations, float *__restrict__ P,
    float *__restrict__ CRLB, float *__restrict__ LL, int nfits)
{
    constexpr int NV = FIT == BAMF_FIT_BASIC ? 4 : (FIT == BAMF_FIT_SIGMAYX ? 6 : 5);
    extern __shared__ float sm[];
    const int npx = sz * sz;
    const int64_t first = (int64_t)blockIdx.x * FITS_PER_BLOCK;
    const int nblk = (int)min((int64_t)FITS_PER_BLOCK, (int64_t)nfits - first);
    /* staged ROIs, then per fit the start-up filter's weight table, then the
     * pixel -> (ii, jj) table (ii << 8 | jj) */
    float *wt = sm + FITS_PER_BLOCK * npx;
    int *pix = (int *)(wt + FITS_PER_BLOCK * (2 * MAXSZ));
    for (int i = threadIdx.x; i < nblk * npx; i += blockDim.x) sm[i] = data[first * npx + i];
    for (int q = threadIdx.x; q < npx; q += blockDim.x) pix[q] = (q / sz) << 8 | (q % sz);
    __syncthreads();
    const int g = threadIdx.x / GL, l = threadIdx.x % GL;
    /* a group past the batch's end fits the block's first ROI again (its
     * lanes take part in the warp's shuffles) and writes nothing */
    const bool active = g < nblk;
    const float *d = sm + (active ? g : 0) * npx;
    const int64_t fit = first + (active ? g : 0);
    float c0 = 0.0f, c1 = 0.0f;
    if (SCMOS) {
        c0 = coords[2 * fit];
        c1 = coords[2 * fit + 1];
    }

    float th[6];
    float maxjump[6] = {1e0f, 1e0f, 1e2f, 2e0f, FIT == BAMF_FIT_SIGMA ? 5e-1f : 1e-1f, 1e-1f};
    /* kernel_CenterofMass2D (GPUgaussLib.cuh:207-227): lane partial sums */
    float tx = 0.0f, ty = 0.0f, ts = 0.0f;
    for (int p = l; p < npx; p += GL) {
        const int ii = pix[p] >> 8, jj = pix[p] & 255;
        const float v = d[sz * jj + ii];
        tx += v * ii;
        ty += v * jj;
        ts += v;
    }
    th[0] = group_sum(tx) / group_sum(ts);
    th[1] = group_sum(ty) / group_sum(ts);
    /* kernel_GaussFMaxMin2D (:230-258): each lane filters its positions with
     * the group's table of the distinct weights */
    const float s_init = FIT == BAMF_FIT_Z ? zp.sx : sigma;
    float *w = wt + g * (2 * MAXSZ);
    {
        const float norm = 1.0f / 2.0f / s_init / s_init;
        for (int q = l - (sz - 1); q <= sz - 1; q += GL) w[q + sz - 1] = expf(-(float)(q * q) * norm);
    }
    __syncwarp();
    float Nmax = 0.0f, MinBG = 10e10f;
    for (int pos = l; pos < npx; pos += GL) {
        const int kk = pix[pos] >> 8, ll = pix[pos] & 255;
        float fp = 0.0f, sum = 0.0f;
        for (int ii = 0; ii < sz; ii++)
            for (int jj = 0; jj < sz; jj++) {
                float ww = w[ii - kk + sz - 1] * w[ll - jj + sz - 1];
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
    th[3] = MinBG;
    if (FIT == BAMF_FIT_Z) {
        th[2] = fmaxf(0.0f, (Nmax - th[3]) * 2 * MLE_PI * zp.sx * zp.sy * sqrtf(2.0f));
        th[4] = 0.0f; /* z0: gaussMLE.m passes zeros */
    } else {
        th[2] = fmaxf(0.0f, (Nmax - th[3]) * 2 * 2 * MLE_PI * sigma * sigma);
        th[4] = sigma;
        th[5] = sigma;
    }

    for (int kk = 0; kk < iterations; kk++) {
        float num[6] = {0, 0, 0, 0, 0, 0}, den[6] = {0, 0, 0, 0, 0, 0};
        for (int p = l; p < npx; p += GL) {
            const int ii = pix[p] >> 8, jj = pix[p] & 255;
            float PSFx, PSFy, du[6], d2u[6];
            pixel<FIT>(ii, jj, th, sigma, zp, &PSFx, &PSFy, du, d2u);
            float model = th[3] + th[2] * PSFx * PSFy;
            float dv = d[sz * jj + ii];
            float cf = 0.0f, df = 0.0f;
            if (SCMOS) {
                int gi = (int)((c1 + jj) * mapsz + c0 + ii);
                gi = min(max(gi, 0), mapsz * mapsz - 1); /* corners outside the map: edge value */
                const float gRp = gmap[gi];
                if (model > 10e-3f) cf = (dv - model) / (model + gRp);
                if (model > 10e-3f) df = (dv + gRp) / ((model + gRp) * (model + gRp));
            } else {
                if (model > 10e-3f) cf = dv / model - 1;
                if (model > 10e-3f) df = dv / (model * model);
            }
            cf = fminf(cf, 10e4f);
            df = fminf(df, 10e4f);
            for (int q = 0; q < NV; q++) {
                num[q] += du[q] * cf;
                den[q] += d2u[q] * cf - (du[q] * du[q]) * df;
            }
        }
        for (int q = 0; q < NV; q++) {
            num[q] = group_sum(num[q]);
            den[q] = group_sum(den[q]);
        }
        th[0] -= fminf(fmaxf(num[0] / den[0], -maxjump[0]), maxjump[0]);
        th[1] -= fminf(fmaxf(num[1] / den[1], -maxjump[1]), maxjump[1]);
        th[2] -= fminf(fmaxf(num[2] / den[2], -th[2]), th[2]);
        th[3] -= fminf(fmaxf(num[3] / den[3], -th[3]), th[3]);
        if (FIT == BAMF_FIT_SIGMA || FIT == BAMF_FIT_SIGMAYX) th[4] -= fminf(fmaxf(num[4] / den[4], -th[4]), th[4]);
        if (FIT == BAMF_FIT_SIGMAYX) th[5] -= fminf(fmaxf(num[5] / den[5], -th[5]), th[5]);
        if (FIT == BAMF_FIT_Z) th[4] -= fminf(fmaxf(num[4] / den[4], -maxjump[4]), maxjump[4]);
        th[2] = fmaxf(th[2], 1.0f);
        th[3] = fmaxf(th[3], 0.01f);
        if (FIT == BAMF_FIT_SIGMA || FIT == BAMF_FIT_SIGMAYX) {
            th[4] = fmaxf(th[4], 0.5f);
            th[4] = fminf(th[4], sz / 2.0f);
        }
        if (FIT == BAMF_FIT_SIGMAYX) {
            th[5] = fmaxf(th[5], 0.5f);
            th[5] = fminf(th[5], sz / 2.0f);
        }
    }
    /* the reference's CRLB / log-likelihood pass uses the variance-gain
     * ratio left from the last pixel of the last iteration, (sz-1, sz-1) */
    float gR = 0.0f;
    if (SCMOS && iterations > 0) {
        int gi = (int)((c1 + (sz - 1)) * mapsz + c0 + (sz - 1));
        gR = gmap[min(max(gi, 0), mapsz * mapsz - 1)];
    }

    /* Fisher information (distinct entries, lane partial sums) and
     * log-likelihood */
    constexpr int NF = NV * (NV + 1) / 2;
    float F[NF];
    for (int q = 0; q < NF; ++q) F[q] = 0.0f;
    float Div = 0.0f;
    for (int p = l; p < npx; p += GL) {
        const int ii = pix[p] >> 8, jj = pix[p] & 255;
        float PSFx, PSFy, du[6];
        pixel<FIT>(ii, jj, th, sigma, zp, &PSFx, &PSFy, du, nullptr);
        float model = th[3] + th[2] * PSFx * PSFy;
        float dv = d[sz * jj + ii];
        float den = SCMOS ? model + gR : model;
        int e = 0;
        for (int a = 0; a < NV; a++)
            for (int b = a; b < NV; b++) F[e++] += du[b] * du[a] / den;
        if (SCMOS) {
            if (model + gR > 0) {
                if (dv + gR > 0)
                    Div += (dv + gR) * logf(model + gR) - model - (dv + gR) * logf(dv + gR) + dv;
                else
                    Div += -model - gR;
            }
        } else if (model > 0) {
            if (dv > 0)
                Div += dv * logf(model) - model - dv * logf(dv) + dv;
            else
                Div += -model;
        }
    }
    for (int q = 0; q < NF; ++q) F[q] = group_sum(F[q]);
    Div = group_sum(Div);
    if (l != 0 || !active) return;
    float M[NV * NV];
    {
        int e = 0;
        for (int a = 0; a < NV; a++)
            for (int b = a; b < NV; b++) {
                M[a * NV + b] = F[e];
                M[b * NV + a] = F[e];
                ++e;
            }
    }
    /* inverse by LU without pivoting (the order of MatInvLib.h:15-75),
     * diagonal only */
    float Minv[NV * NV], yy[NV], tmp1 = 0.0f;
    for (int jj = 0; jj < NV; jj++) {
        for (int ii = 1; ii <= jj; ii++) {
            for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * NV] * M[q + jj * NV];
            M[ii + jj * NV] -= tmp1;
            tmp1 = 0.0f;
        }
        for (int ii = jj + 1; ii < NV; ii++) {
            if (jj > 0) {
                for (int q = 0; q <= jj - 1; q++) tmp1 += M[ii + q * NV] * M[q + jj * NV];
                M[ii + jj * NV] = (1 / M[jj + jj * NV]) * (M[ii + jj * NV] - tmp1);
                tmp1 = 0.0f;
            } else {
                M[ii + jj * NV] = (1 / M[jj + jj * NV]) * M[ii + jj * NV];
            }
        }
    }
    for (int num = 0; num < NV; num++) {
        yy[0] = num == 0 ? 1.0f : 0.0f;
        for (int ii = 1; ii < NV; ii++) {
            float b = ii == num ? 1.0f : 0.0f;
            for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * NV] * yy[q];
            yy[ii] = b - tmp1;
            tmp1 = 0.0f;
        }
        Minv[NV - 1 + num * NV] = yy[NV - 1] / M[(NV - 1) + (NV - 1) * NV];
        for (int ii = NV - 2; ii >= 0; ii--) {
            for (int q = ii + 1; q < NV; q++) tmp1 += M[ii + q * NV] * Minv[q + num * NV];
            Minv[ii + num * NV] = (1 / M[ii + ii * NV]) * (yy[ii] - tmp1);
            tmp1 = 0.0f;
        }
    }
    for (int k = 0; k < NV; k++) {
        P[(int64_t)nfits * k + fit] = th[k];
        CRLB[(int64_t)nfits * k + fit] = Minv[k * NV + k];
    }
    LL[fit] = Div;
}

template <int FIT, bool SCMOS>
cudaError_t launch(const float *rois, int sz, int nfits, float sigma, const ZPar &zp, const float *coords,
                   const float *gmap, int mapsz, int iterations, float *P, float *C, float *L, cudaStream_t s)
{
    size_t smem = ((size_t)FITS_PER_BLOCK * (sz * sz + 2 * MAXSZ) + (size_t)sz * sz) * sizeof(float);
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(mle_fit_kernel<FIT, SCMOS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int blocks = (nfits + FITS_PER_BLOCK - 1) / FITS_PER_BLOCK;
    mle_fit_kernel<FIT, SCMOS><<<blocks, GL * FITS_PER_BLOCK, smem, s>>>(rois, sigma, zp, coords, gmap, mapsz, sz,
                                                                         iterations, P, C, L, nfits);
    return cudaGetLastError();
}

}  // namespace

extern "C" int bamf_gauss_mle_nparams(int fit_type)
{
    switch (fit_type) {
    case BAMF_FIT_BASIC: return 4;
    case BAMF_FIT_SIGMA: return 5;
    case BAMF_FIT_Z: return 5;
    case BAMF_FIT_SIGMAYX: return 6;
    default: return -1;
    }
}

extern "C" bamf_status bamf_gauss_mle_fit_device(const float *rois, int sz, int nfits, int fit_type, float psf_sigma,
                                                 const bamf_zfit *zfit, const float *box_corners,
                                                 const float *var_gain_map, int map_size, int iterations,
                                                 float *params, float *crlb, float *loglik, void *stream)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0 || iterations < 0) return BAMF_ERR_INVALID_ARG;
    if (bamf_gauss_mle_nparams(fit_type) < 0) return BAMF_ERR_INVALID_ARG;
    if (fit_type == BAMF_FIT_Z && !zfit) return BAMF_ERR_INVALID_ARG;
    const bool scmos = var_gain_map != nullptr;
    if (scmos && (!box_corners || map_size < 1)) return BAMF_ERR_INVALID_ARG;
    if (sz > MAXSZ) return BAMF_ERR_TOO_LARGE;
    if (nfits == 0) return BAMF_OK;
    if (!scmos && fit_type == BAMF_FIT_BASIC)
        return bamf_gauss_mle_device(rois, sz, nfits, psf_sigma, iterations, params, crlb, loglik, stream);
    ZPar zp = {0, 0, 0, 0, 0, 0, 0, 1};
    if (zfit) zp = {zfit->sigma_x, zfit->sigma_y, zfit->Ax, zfit->Ay, zfit->Bx, zfit->By, zfit->gamma, zfit->d};
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
#define BAMF_FIT_CASE(F)                                                                                          \
    e = scmos ? launch<F, true>(rois, sz, nfits, psf_sigma, zp, box_corners, var_gain_map, map_size, iterations,  \
                                params, crlb, loglik, s)                                                          \
              : launch<F, false>(rois, sz, nfits, psf_sigma, zp, nullptr, nullptr, 0, iterations, params, crlb,   \
                                 loglik, s)
    switch (fit_type) {
    case BAMF_FIT_BASIC: BAMF_FIT_CASE(BAMF_FIT_BASIC); break;
    case BAMF_FIT_SIGMA: BAMF_FIT_CASE(BAMF_FIT_SIGMA); break;
    case BAMF_FIT_Z: BAMF_FIT_CASE(BAMF_FIT_Z); break;
    default: BAMF_FIT_CASE(BAMF_FIT_SIGMAYX); break;
    }
#undef BAMF_FIT_CASE
    return e == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_gauss_mle_fit_host(const float *rois, int sz, int nfits, int fit_type, float psf_sigma,
                                               const bamf_zfit *zfit, const float *box_corners,
                                               const float *var_gain_map, int map_size, int iterations,
                                               float *params, float *crlb, float *loglik)
{
    const int np = bamf_gauss_mle_nparams(fit_type);
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0 || np < 0) return BAMF_ERR_INVALID_ARG;
    if (var_gain_map && (!box_corners || map_size < 1)) return BAMF_ERR_INVALID_ARG;
    if (sz > MAXSZ) return BAMF_ERR_TOO_LARGE;
    if (nfits == 0) return BAMF_OK;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    float *dr = nullptr, *dp = nullptr, *dc = nullptr, *dl = nullptr, *dco = nullptr, *dm = nullptr;
    const size_t nin = (size_t)nfits * sz * sz, nout = (size_t)nfits * np;
    bamf_status st = BAMF_OK;
    if (cudaMalloc(&dr, nin * 4) != cudaSuccess || cudaMalloc(&dp, nout * 4) != cudaSuccess ||
        cudaMalloc(&dc, nout * 4) != cudaSuccess || cudaMalloc(&dl, (size_t)nfits * 4) != cudaSuccess)
        st = BAMF_ERR_CUDA;
    if (!st && var_gain_map &&
        (cudaMalloc(&dco, (size_t)nfits * 2 * 4) != cudaSuccess ||
         cudaMalloc(&dm, (size_t)map_size * map_size * 4) != cudaSuccess))
        st = BAMF_ERR_CUDA;
    if (!st && cudaMemcpy(dr, rois, nin * 4, cudaMemcpyHostToDevice) != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st && var_gain_map &&
        (cudaMemcpy(dco, box_corners, (size_t)nfits * 2 * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
         cudaMemcpy(dm, var_gain_map, (size_t)map_size * map_size * 4, cudaMemcpyHostToDevice) != cudaSuccess))
        st = BAMF_ERR_CUDA;
    if (!st)
        st = bamf_gauss_mle_fit_device(dr, sz, nfits, fit_type, psf_sigma, zfit, dco, dm, map_size, iterations, dp,
                                       dc, dl, nullptr);
    if (!st && cudaDeviceSynchronize() != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st && (cudaMemcpy(params, dp, nout * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(crlb, dc, nout * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(loglik, dl, (size_t)nfits * 4, cudaMemcpyDeviceToHost) != cudaSuccess))
        st = BAMF_ERR_CUDA;
    void *ps[] = {dr, dp, dc, dl, dco, dm};
    for (void *q : ps)
        if (q) cudaFree(q);
    if (st) cudaGetLastError();
    return st;
}
