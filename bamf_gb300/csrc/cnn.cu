/*
 * cnn.cu - the learned birth proposal (include/bamf_cnn.h): synthetic ROI
 * generator, the network's forward and backward kernels, Adam, a CUDA-graph
 * training step, and inference into the sampler's LEARNED birth tables.
 *
 * Layouts.  Activations are channels-last BF16, [roi][p][32] with pixel
 * p = y + 16 x.  The three 32 -> 32 convolutions (forward and input
 * gradient) run on the 5th-generation tensor cores (tcgen05.mma from
 * shared-memory descriptors into TMEM, conv_tc_kernel): per ROI an implicit
 * GEMM with M = 256 pixels (two tiles of 128), N = 32, K = 9 taps x 32
 * channels.  The input gradient of a convolution is the same kernel run with
 * the taps flipped and the channel roles swapped (packed once per step).
 * The weight gradient is a GEMM with K = the pixels of every ROI of the
 * CTA, also on tcgen05, with MN-major operands so that the channels-last
 * activations stage without a transpose (conv_dw_tc_kernel).
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "bamf.h"
#include "bamf_cnn.h"
#include "bamf_philox.h"
#include "tc_ptx.cuh"

namespace {

constexpr int S = BAMF_CNN_SIDE;  /* 16 */
constexpr int NPX = S * S;        /* 256 */
constexpr int CH = BAMF_CNN_CH;   /* 32 */
constexpr int PS = S + 2;         /* padded side */
constexpr int NC = BAMF_CNN_COUNTS;
constexpr int NSUB = 16;
constexpr int MAX_BATCH = 4096;

/* parameter offsets */
constexpr int O_W1 = 0, O_B1 = 288, O_W2 = 320, O_B2 = 9536, O_W3 = 9568, O_B3 = 18784, O_W4 = 18816,
              O_B4 = 28032, O_WL = 28064, O_BL = 28576, O_WC = 28592, O_BC = 28944, NPARAM = 28955;
static_assert(NPARAM == BAMF_CNN_NPARAM, "parameter count");
static_assert(O_B1 == O_W1 + 288 && O_BC + NC == NPARAM, "conv1 block and head layout");
constexpr int HEAD_NPARAM = NPARAM - O_WL; /* WL, BL, WC, BC: the heads' parameters, contiguous */
static_assert(O_BL == O_WL + NSUB * CH && O_WC == O_BL + NSUB && O_BC == O_WC + NC * CH, "head layout");
constexpr int C1_NPARAM = O_W2;            /* W1, B1 */
constexpr int HS = CH + 4;                 /* head kernel: floats per pixel row of H (16-byte rows) */
/* the WC part of ROI r's head-gradient row */
__device__ __forceinline__ float *row_wc(float *rows, int r) { return rows + (size_t)r * HEAD_NPARAM + (O_WC - O_WL); }
constexpr int O_W[3] = {O_W2, O_W3, O_W4};
constexpr int O_B[3] = {O_B2, O_B3, O_B4};
constexpr int PKT = 9 * CH * CH; /* tensor-core operand weights of one layer */

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ float u01(uint32_t w)
{
    return ((float)(w >> 8) + 0.5f) * (1.0f / 16777216.0f); /* (0, 1) */
}

/* ------------------------------------------------------------- generator */
/* Poisson(lam): multiplication method below 10, else the PTRS transformed
 * rejection of W. Hoermann, "The transformed rejection method for generating
 * Poisson random variables", Insurance: Mathematics and Economics 12 (1993).
 * Uniforms come from the Philox blocks (c0, c1, c2, j) of key (k0, k1). */
__device__ int poisson_draw(float lam, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t k0, uint32_t k1)
{
    if (!(lam > 0.0f)) return 0;
    if (lam < 10.0f) {
        float L = expf(-lam), prod = 1.0f;
        int n = 0;
        for (uint32_t j = 0; j < 16; ++j) {
            bamf_philox_block b = bamf_philox4x32_10(c0, c1, c2, j, k0, k1);
            for (int w = 0; w < 4; ++w) {
                prod *= u01(b.v[w]);
                if (prod <= L) return n;
                ++n;
            }
        }
        return n;
    }
    const float slam = sqrtf(lam), loglam = logf(lam);
    const float b = 0.931f + 2.53f * slam;
    const float a = -0.059f + 0.02483f * b;
    const float invalpha = 1.1239f + 1.1328f / (b - 3.4f);
    const float vr = 0.9277f - 3.6224f / (b - 2.0f);
    for (uint32_t j = 0; j < 32; ++j) {
        bamf_philox_block blk = bamf_philox4x32_10(c0, c1, c2, j, k0, k1);
        for (int h = 0; h < 2; ++h) {
            float U = u01(blk.v[2 * h]) - 0.5f;
            float V = u01(blk.v[2 * h + 1]);
            float us = 0.5f - fabsf(U);
            float k = floorf((2.0f * a / us + b) * U + lam + 0.43f);
            if (us >= 0.07f && V <= vr) return (int)k;
            if (k < 0.0f || (us < 0.013f && V > us)) continue;
            if (logf(V) + logf(invalpha) - logf(a / (us * us) + b) <= -lam + k * loglam - lgammaf(k + 1.0f))
                return (int)k;
        }
    }
    return (int)floorf(lam + 0.5f); /* not reached in practice (acceptance > 0.9 per round) */
}

__global__ void synth_kernel(bamf_synth_params sp, uint32_t seed, uint64_t first, const int *step_dev,
                             int batch, int n, float *__restrict__ data, int32_t *__restrict__ n_em,
                             float *__restrict__ xyi)
{
    __shared__ float ex[BAMF_SYNTH_NMAX], ey[BAMF_SYNTH_NMAX], ei[BAMF_SYNTH_NMAX];
    __shared__ int ne;
    int r = blockIdx.x;
    if (r >= n) return;
    uint64_t k = (step_dev ? (uint64_t)(*step_dev) * (uint64_t)batch : first) + (uint64_t)r;
    uint32_t klo = (uint32_t)k, khi = (uint32_t)(k >> 32);
    const uint32_t K1 = 0x6a09e667u ^ khi;
    int t = threadIdx.x;
    if (t == 0) {
        float L = expf(-sp.mean_n), prod = 1.0f;
        int cnt = 0;
        bool done = false;
        for (uint32_t j = 0; j < 16 && !done; ++j) {
            bamf_philox_block b = bamf_philox4x32_10(klo, 0u, j, 0u, seed, K1);
            for (int w = 0; w < 4; ++w) {
                prod *= u01(b.v[w]);
                if (prod <= L) {
                    done = true;
                    break;
                }
                ++cnt;
            }
        }
        ne = min(cnt, BAMF_SYNTH_NMAX);
    }
    if (t < BAMF_SYNTH_NMAX) {
        bamf_philox_block b = bamf_philox4x32_10(klo, 1u, (uint32_t)t, 0u, seed, K1);
        ex[t] = (float)S * u01(b.v[0]);
        ey[t] = (float)S * u01(b.v[1]);
        float z = sqrtf(-2.0f * logf(u01(b.v[2]))) * cospif(2.0f * u01(b.v[3]));
        ei[t] = expf(logf(sp.i_median) + sp.i_logsd * z);
    }
    __syncthreads();
    const int nn = ne;
    if (t < BAMF_SYNTH_NMAX) {
        float *o = xyi + ((size_t)r * BAMF_SYNTH_NMAX + t) * 3;
        bool on = t < nn;
        o[0] = on ? ex[t] : 0.0f;
        o[1] = on ? ey[t] : 0.0f;
        o[2] = on ? ei[t] : 0.0f;
    }
    if (t == 0) n_em[r] = nn;
    int x = t / S, y = t - (t / S) * S;
    const float c = 1.0f / (sqrtf(2.0f) * sp.sigma);
    float bgv = sp.bg;
    if (sp.bg_max > sp.bg) {
        bamf_philox_block bb = bamf_philox4x32_10(klo, 3u, 0u, 0u, seed, K1);
        bgv = sp.bg + (sp.bg_max - sp.bg) * u01(bb.v[0]);
    }
    float lam = bgv;
    for (int e = 0; e < nn; ++e) {
        float sx = 0.5f * (erff(((float)x - ex[e] + 1.0f) * c) - erff(((float)x - ex[e]) * c));
        float sy = 0.5f * (erff(((float)y - ey[e] + 1.0f) * c) - erff(((float)y - ey[e]) * c));
        lam += ei[e] * sx * sy;
    }
    data[(size_t)r * NPX + t] = (float)poisson_draw(lam, klo, 2u, (uint32_t)t, seed, K1);
}

/* -------------------------------------------------------- weight packing */
/* The B operands of the 32 -> 32 convolutions for the tensor cores, per
 * layer [tap][ci group g][n][8] BF16 (K-major core matrices: 8 n x 8 k):
 * forward Wf: B[n = co][k = ci] = W_l[co][ci][tap]; input gradient Wb:
 * B[n = ci][k = co] = W_l[co][ci][8 - tap]. */
__global__ void pack_kernel(const float *__restrict__ P, bf16 *__restrict__ Wf, bf16 *__restrict__ Wb)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * PKT) return;
    int l = i / PKT, rem = i - l * PKT;
    int tap = rem / (CH * CH), nk = rem - tap * CH * CH;
    int nn = nk / CH, kk = nk - nn * CH;
    const float *W = P + (l == 0 ? O_W2 : (l == 1 ? O_W3 : O_W4));
    const int o = l * PKT + tap * CH * CH + (kk >> 3) * (CH * 8) + nn * 8 + (kk & 7);
    Wf[o] = __float2bfloat16_rn(W[(nn * CH + kk) * 9 + tap]);
    Wb[o] = __float2bfloat16_rn(W[(kk * CH + nn) * 9 + (8 - tap)]);
}

/* --------------------------------------------------------------- conv1 */
/* x0 normalisation and the 1 -> 32 convolution (FP32), one CTA per ROI. */
__global__ void conv1_fwd_kernel(const float *__restrict__ data, int n, const float *__restrict__ P,
                                 float *__restrict__ x0, bf16 *__restrict__ a1)
{
    __shared__ float xp[PS * PS];
    __shared__ float w[288 + 32];
    __shared__ float red[8];
    int r = blockIdx.x, t = threadIdx.x;
    if (r >= n) return;
    for (int i = t; i < 320; i += blockDim.x) w[i] = P[O_W1 + i];
    for (int i = t; i < PS * PS; i += blockDim.x) xp[i] = 0.0f;
    float v = sqrtf(fmaxf(data[(size_t)r * NPX + t], 0.0f) + 0.375f);
    float s = v;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((t & 31) == 0) red[t >> 5] = s;
    __syncthreads();
    float mean = 0.0f;
    for (int k = 0; k < 8; ++k) mean += red[k];
    mean *= (1.0f / NPX);
    float xv = (v - mean) * 0.25f;
    int x = t / S, y = t - (t / S) * S;
    xp[(x + 1) * PS + (y + 1)] = xv;
    if (x0) x0[(size_t)r * NPX + t] = xv;
    __syncthreads();
    float in[9];
    for (int kx = 0; kx < 3; ++kx)
        for (int ky = 0; ky < 3; ++ky) in[kx * 3 + ky] = xp[(x + kx) * PS + (y + ky)];
    __align__(16) bf16 o[CH];
    for (int co = 0; co < CH; ++co) {
        float z = w[288 + co];
        for (int tp = 0; tp < 9; ++tp) z += w[co * 9 + tp] * in[tp];
        o[co] = __float2bfloat16_rn(fmaxf(z, 0.0f));
    }
    uint4 *dst = (uint4 *)(a1 + ((size_t)r * NPX + t) * CH);
    const uint4 *src = (const uint4 *)o;
    for (int q = 0; q < 4; ++q) dst[q] = src[q];
}

/* dW1, db1 from dz1 (= dL/d pre-activation of conv1) and x0: each CTA's
 * sums over its ROIs into row blockIdx.x of `rows` (C1_NPARAM floats).  Warp w
 * owns output channels 4w .. 4w + 3 (all 9 taps and the bias), lane l the
 * pixels l + 32 i: per pixel 9 neighbours and 4 dz values from shared
 * memory feed 40 register accumulators, kept over all the CTA's ROIs and
 * reduced over the warp once at the end. */
__global__ void __launch_bounds__(256) conv1_bwd_kernel(const float *__restrict__ x0, const bf16 *__restrict__ dz1,
                                                        int n, float *__restrict__ rows)
{
    __shared__ float xp[PS * PS];
    __shared__ float dz[NPX * (CH + 1)];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    float acc[4][9], accb[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        accb[j] = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[j][k] = 0.0f;
    }
    for (int i = t; i < PS * PS; i += blockDim.x) xp[i] = 0.0f;
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        __syncthreads();
        {
            const int x = t / S, y = t - (t / S) * S;
            xp[(x + 1) * PS + (y + 1)] = x0[(size_t)r * NPX + t];
            const uint4 *src = (const uint4 *)(dz1 + ((size_t)r * NPX + t) * CH);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 u = src[q];
                const __nv_bfloat162 *b = (const __nv_bfloat162 *)&u;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float2 f = __bfloat1622float2(b[e]);
                    dz[t * (CH + 1) + 8 * q + 2 * e] = f.x;
                    dz[t * (CH + 1) + 8 * q + 2 * e + 1] = f.y;
                }
            }
        }
        __syncthreads();
#pragma unroll 2
        for (int i = 0; i < NPX / 32; ++i) {
            const int p = lane + 32 * i, x = p >> 4, y = p & 15;
            float nb[9];
#pragma unroll
            for (int kx = 0; kx < 3; ++kx)
#pragma unroll
                for (int ky = 0; ky < 3; ++ky) nb[kx * 3 + ky] = xp[(x + kx) * PS + (y + ky)];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float d = dz[p * (CH + 1) + 4 * warp + j];
                accb[j] += d;
#pragma unroll
                for (int k = 0; k < 9; ++k) acc[j][k] += d * nb[k];
            }
        }
    }
    float *row = rows + (size_t)blockIdx.x * C1_NPARAM;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            float v = acc[j][k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) row[(4 * warp + j) * 9 + k] = v;
        }
        float v = accb[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) row[288 + 4 * warp + j] = v;
    }
}

/* -------------------------------------------------- 32 -> 32 convolution */
/* MODE 0: out = relu(conv(in, W) + bias).  MODE 1 (input gradient):
 * out = conv(in, W) * (mask > 0).  On the 5th-generation tensor cores: per
 * ROI an implicit GEMM D[pixel][co] = sum over 9 taps of A_tap[pixel][ci]
 * B_tap[co][ci], M = 256 pixels as two tiles of 128, N = 32, K = 32 per tap
 * as two MMAs of 16: 36 tcgen05.mma (BF16 x BF16 -> FP32) issued by one
 * thread into TMEM (64 columns), completion through an mbarrier, epilogue
 * from tcgen05.ld.
 *
 * A operands straight from shared memory: the ROI is staged as three copies
 * shifted by ky - 1 along y, each [ci group g][padded x 0..17][y 0..15][8 ci]
 * BF16, so that for tap (kx, ky) the 128 rows of M tile t (pixels p = 128 t
 * + m, x = p / 16, y = p mod 16) are 16-byte rows at consecutive addresses
 * from (8 t + kx) * 16 rows into copy ky: K-major core matrices with SBO =
 * 128 B and LBO = one ci group.  Borders stay zero.  One ROI per iteration
 * of a persistent CTA of 128 threads (thread m owns pixels m and 128 + m in
 * the epilogue).  The mbarrier wait is bounded; a timeout is recorded in
 * *status and the kernel frees its TMEM and returns. */
constexpr int TC_GSTRIDE = PS * S * 16;            /* bytes of one ci group of one copy */
constexpr int TC_COPY = 4 * TC_GSTRIDE;            /* bytes of one shifted copy */
constexpr size_t SMEM_TC = (size_t)PKT * 2 + 3 * TC_COPY + 16;
constexpr uint32_t TC_IDESC = bamf::tc::idesc_bf16_f32(128, 32);

template <int MODE>
__global__ void __launch_bounds__(128) conv_tc_kernel(const bf16 *__restrict__ in, const bf16 *__restrict__ Wt,
                                                      const float *__restrict__ bias,
                                                      const bf16 *__restrict__ mask, bf16 *__restrict__ out, int n,
                                                      int *__restrict__ status)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *Ws = smem_raw;                    /* [9][4][32][8] bf16 */
    unsigned char *Cp = smem_raw + PKT * 2;          /* 3 copies */
    uint64_t *mbar = (uint64_t *)(Cp + 3 * TC_COPY);
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) bamf::tc::tmem_alloc(&tslot, 64);
    {
        const uint4 *src = (const uint4 *)Wt;
        uint4 *dst = (uint4 *)Ws;
        for (int i = t; i < PKT * 2 / 16; i += blockDim.x) dst[i] = src[i];
        const uint4 z = make_uint4(0, 0, 0, 0);
        uint4 *cc = (uint4 *)Cp;
        for (int i = t; i < 3 * TC_COPY / 16; i += blockDim.x) cc[i] = z;
    }
    if (t == 0) bamf::tc::mbar_init(mbar, 1);
    bamf::tc::fence_before_sync();
    __syncthreads();
    bamf::tc::fence_after_sync();
    const uint32_t tbase = tslot;
    const uint32_t ws_addr = bamf::tc::smem_addr(Ws), cp_addr = bamf::tc::smem_addr(Cp);
    uint32_t phase = 0;
    bool alive = true;
    /* each thread carries 8 of the ROI's 1024 16-byte chunks (8 channels of
     * one pixel): pixels (t & 7) + 8 (t >> 5) + 32 k, channel group
     * (t >> 3) & 3, so that the 8 lanes of a 16-byte store phase write 8
     * consecutive pixels of one group (one bank group each); the next ROI's
     * chunks are loaded while the current ROI's MMAs run, and staged once
     * they completed */
    constexpr int CPT = NPX * 4 / 128;
    const int cg = (t >> 3) & 3, p0 = (t & 7) + 8 * (t >> 5);
    uint4 pre[CPT];
    auto load = [&](int r) {
        const uint4 *src = (const uint4 *)(in + (size_t)r * NPX * CH);
#pragma unroll
        for (int k = 0; k < CPT; ++k) pre[k] = src[(p0 + 32 * k) * 4 + cg];
    };
    /* each chunk goes to the three shifted copies where it lands inside */
    auto stage = [&]() {
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            const int p = p0 + 32 * k, g = cg, x = p >> 4, y = p & 15;
#pragma unroll
            for (int ky = 0; ky < 3; ++ky) {
                const int yo = y - ky + 1;
                if (yo >= 0 && yo < S)
                    *(uint4 *)(Cp + ky * TC_COPY + g * TC_GSTRIDE + ((x + 1) * S + yo) * 16) = pre[k];
            }
        }
    };
    if (blockIdx.x < n) {
        load(blockIdx.x);
        stage();
    }
    for (int r = blockIdx.x; r < n && alive; r += gridDim.x) {
        bamf::tc::fence_proxy_async();
        bamf::tc::fence_before_sync();
        __syncthreads();
        bamf::tc::fence_after_sync();
        if (t == 0) {
            uint32_t acc = 0;
#pragma unroll 1
            for (int mt = 0; mt < 2; ++mt) {
                acc = 0;
                for (int tap = 0; tap < 9; ++tap) {
                    const int kx = tap / 3, ky = tap - kx * 3;
                    for (int cb = 0; cb < 2; ++cb) {
                        const uint32_t a = cp_addr + ky * TC_COPY + (2 * cb) * TC_GSTRIDE + (8 * mt + kx) * S * 16;
                        const uint32_t b = ws_addr + tap * (CH * CH * 2) + (2 * cb) * (CH * 16);
                        bamf::tc::mma_bf16(tbase + 32 * mt, bamf::tc::smem_desc(a, TC_GSTRIDE, 128),
                                           bamf::tc::smem_desc(b, CH * 16, 128), TC_IDESC, acc);
                        acc = 1;
                    }
                }
            }
            bamf::tc::commit(mbar);
        }
        const int rn = r + gridDim.x;
        if (rn < n) load(rn);
        /* MODE 1: this thread's two pixels of the ReLU mask, loaded while
         * the MMAs run */
        uint4 mk[2][4];
        if (MODE == 1) {
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const uint4 *ms = (const uint4 *)(mask + ((size_t)r * NPX + 128 * mt + t) * CH);
#pragma unroll
                for (int q = 0; q < 4; ++q) mk[mt][q] = ms[q];
            }
        }
        const bool ok = bamf::tc::mbar_wait(mbar, phase, 1u << 24);
        phase ^= 1u;
        bamf::tc::fence_after_sync();
        if (!ok) {
            if (t == 0) atomicExch(status, 1);
            alive = false;
        } else {
#pragma unroll 1
            for (int mt = 0; mt < 2; ++mt) {
                float v[32];
                bamf::tc::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + 32 * mt, v);
                const int p = 128 * mt + t;
                const size_t off = ((size_t)r * NPX + p) * CH;
                __align__(16) __nv_bfloat162 o[16];
                if (MODE == 0) {
#pragma unroll
                    for (int c = 0; c < 16; ++c)
                        o[c] = __floats2bfloat162_rn(fmaxf(v[2 * c] + bias[2 * c], 0.0f),
                                                     fmaxf(v[2 * c + 1] + bias[2 * c + 1], 0.0f));
                } else {
                    __align__(16) uint4 m4[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) m4[q] = mt == 0 ? mk[0][q] : mk[1][q];
                    const __nv_bfloat162 *m2 = (const __nv_bfloat162 *)m4;
#pragma unroll
                    for (int c = 0; c < 16; ++c)
                        o[c] = __floats2bfloat162_rn(__bfloat162float(m2[c].x) > 0.0f ? v[2 * c] : 0.0f,
                                                     __bfloat162float(m2[c].y) > 0.0f ? v[2 * c + 1] : 0.0f);
                }
                uint4 *dst = (uint4 *)(out + off);
#pragma unroll
                for (int q = 0; q < 4; ++q) dst[q] = ((uint4 *)o)[q];
            }
        }
        bamf::tc::fence_before_sync();
        __syncthreads(); /* TMEM read and copies consumed before the next ROI */
        bamf::tc::fence_after_sync();
        alive = __syncthreads_and(alive);
        if (alive && rn < n) stage();
    }
    bamf::tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) bamf::tc::tmem_dealloc(tbase, 64);
}

/* Weight and bias gradient of a 32 -> 32 convolution on the tensor cores:
 * dW[co][ci][tap] += sum over ROIs and pixels p of act[p + tap][ci] dz[p][co]
 * with tap = 3 kx + ky the shift (kx - 1, ky - 1) in (x, y).  Substituting
 * q = p + 16 (kx - 1) (the x shift moves a pixel index by 16),
 *   D[(ky, ci)][(kx, co)] = sum over q in [0, 256) of
 *                           A[(ky, ci)][q] * B[(kx, co)][q],
 *   A[(ky, ci)][q] = act[q + ky - 1][ci] (zero where y(q) + ky - 1 leaves
 *                    the ROI),
 *   B[(kx, co)][q] = dz[q - 16 (kx - 1)][co] (zero outside the ROI),
 * an M = 128 (96 rows (ky, ci), the last 32 rows ignored) x N = 96 x K = 256
 * GEMM per ROI: 16 tcgen05.mma of K = 16, accumulated in TMEM over all ROIs
 * of the CTA (column 32 kx + co).
 *
 * Both operands MN-major, so that a 16-byte chunk of the channels-last
 * tensors (8 channels of one pixel) is one row of a core matrix and staging
 * is plain 16-byte copies: A as three y-shifted copies of act, B as three
 * x-shifted copies of dz, core matrix (k group j, row block 4 s + g) at
 * j * 1536 + (4 s + g) * 128 (s = ky for A, kx for B).  The ignored rows
 * 96..127 of A read the next k group's rows (in bounds: B follows A).  One
 * ROI per iteration of a persistent CTA of 128 threads, the next ROI's
 * chunks loaded into registers while the MMAs run; the bias gradient (sum of
 * dz over pixels) is formed from the staged chunks.  A lane's chunks are
 * pixel (t & 7) + 8 (t >> 5) + 32 k, channel group (t >> 3) & 3: the 8 lanes
 * of a 16-byte store phase write 8 consecutive pixels of one block, one
 * shared-memory bank group each.  Each CTA writes its partial sums (D, then
 * the 32 bias sums) to its own slice of `part`, coalesced; dw_reduce_kernel
 * adds the slices in a fixed order (no atomics, the same bits every run).
 * The mbarrier wait is bounded; a timeout is recorded in *status, the CTA
 * writes zeros, frees its TMEM and returns. */
constexpr int DW_KS = 12 * 128;                /* bytes of one k group (8 pixels) */
constexpr int DW_PART = 96 * 96 + CH;          /* floats of one CTA's partial sums */
constexpr int DW_ABYTES = 32 * DW_KS;          /* 256 pixels */
constexpr size_t SMEM_DW = (size_t)2 * DW_ABYTES + 16;
constexpr uint32_t DW_IDESC = bamf::tc::idesc_bf16_f32_mn(128, 96);

__global__ void __launch_bounds__(128) conv_dw_tc_kernel(const bf16 *__restrict__ act, const bf16 *__restrict__ dz,
                                                         int n, float *__restrict__ part, int *__restrict__ status)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *As = smem_raw;
    unsigned char *Bs = smem_raw + DW_ABYTES;
    uint64_t *mbar = (uint64_t *)(Bs + DW_ABYTES);
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) bamf::tc::tmem_alloc(&tslot, 128);
    {
        const uint4 z = make_uint4(0, 0, 0, 0);
        uint4 *dst = (uint4 *)smem_raw;
        for (int i = t; i < 2 * DW_ABYTES / 16; i += blockDim.x) dst[i] = z;
    }
    if (t == 0) bamf::tc::mbar_init(mbar, 1);
    bamf::tc::fence_before_sync();
    __syncthreads();
    bamf::tc::fence_after_sync();
    const uint32_t tbase = tslot;
    const uint32_t a_addr = bamf::tc::smem_addr(As), b_addr = bamf::tc::smem_addr(Bs);
    /* each thread carries 8 of the ROI's 1024 chunks of act and of dz */
    constexpr int CPT = NPX * 4 / 128;
    const int g = (t >> 3) & 3, p0 = (t & 7) + 8 * (t >> 5);
    uint4 pa[CPT], pd[CPT];
    float bsum[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) bsum[c] = 0.0f;
    auto load = [&](int r) {
        const uint4 *sa = (const uint4 *)(act + (size_t)r * NPX * CH);
        const uint4 *sd = (const uint4 *)(dz + (size_t)r * NPX * CH);
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            pa[k] = sa[(p0 + 32 * k) * 4 + g];
            pd[k] = sd[(p0 + 32 * k) * 4 + g];
        }
    };
    auto stage = [&]() {
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            const int p = p0 + 32 * k, y = p & 15;
#pragma unroll
            for (int sh = 0; sh < 3; ++sh) {
                const int yq = y - sh + 1, qa = p - sh + 1; /* A[(sh, .)][qa] = act[p] */
                if (yq >= 0 && yq < S)
                    *(uint4 *)(As + (qa >> 3) * DW_KS + (4 * sh + g) * 128 + (qa & 7) * 16) = pa[k];
                const int qb = p + 16 * (sh - 1); /* B[(sh, .)][qb] = dz[p] */
                if (qb >= 0 && qb < NPX)
                    *(uint4 *)(Bs + (qb >> 3) * DW_KS + (4 * sh + g) * 128 + (qb & 7) * 16) = pd[k];
            }
            const __nv_bfloat162 *h = (const __nv_bfloat162 *)&pd[k];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float2 f = __bfloat1622float2(h[c]);
                bsum[2 * c] += f.x;
                bsum[2 * c + 1] += f.y;
            }
        }
    };
    bool alive = true, first = true;
    uint32_t phase = 0;
    if (blockIdx.x < n) {
        load(blockIdx.x);
        stage();
    }
    for (int r = blockIdx.x; r < n && alive; r += gridDim.x) {
        bamf::tc::fence_proxy_async();
        bamf::tc::fence_before_sync();
        __syncthreads();
        bamf::tc::fence_after_sync();
        if (t == 0) {
#pragma unroll 1
            for (int sk = 0; sk < 16; ++sk)
                bamf::tc::mma_bf16(tbase, bamf::tc::smem_desc(a_addr + 2 * sk * DW_KS, DW_KS, 128),
                                   bamf::tc::smem_desc(b_addr + 2 * sk * DW_KS, DW_KS, 128), DW_IDESC,
                                   (first && sk == 0) ? 0u : 1u);
            bamf::tc::commit(mbar);
        }
        first = false;
        const int rn = r + gridDim.x;
        if (rn < n) load(rn);
        const bool ok = bamf::tc::mbar_wait(mbar, phase, 1u << 24);
        phase ^= 1u;
        bamf::tc::fence_after_sync();
        if (!ok) {
            if (t == 0) atomicExch(status, 1);
            alive = false;
        }
        bamf::tc::fence_before_sync();
        __syncthreads(); /* the MMAs have read the tiles before they are restaged */
        bamf::tc::fence_after_sync();
        alive = __syncthreads_and(alive);
        if (alive && rn < n) stage();
    }
    if (blockIdx.x < n) {
        float *mine = part + (size_t)blockIdx.x * DW_PART;
        if (warp < 3) {
            /* warp ky, lane ci: D[(ky, ci)][(kx, co)] in column 32 kx + co,
             * stored at (32 kx + co) * 96 + 32 ky + ci */
#pragma unroll 1
            for (int kx = 0; kx < 3; ++kx) {
                float v[32];
                if (alive) {
                    bamf::tc::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + 32 * kx, v);
                } else {
#pragma unroll
                    for (int co = 0; co < CH; ++co) v[co] = 0.0f;
                }
#pragma unroll
                for (int co = 0; co < CH; ++co) mine[(32 * kx + co) * 96 + t] = v[co];
            }
        }
        /* bias: lanes with equal (lane >> 3) hold the same 8 channels */
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            float v = bsum[c];
            v += __shfl_xor_sync(0xffffffffu, v, 1);
            v += __shfl_xor_sync(0xffffffffu, v, 2);
            v += __shfl_xor_sync(0xffffffffu, v, 4);
            bsum[c] = v;
        }
        __shared__ float bred[4][CH];
        if ((t & 7) == 0)
#pragma unroll
            for (int c = 0; c < 8; ++c) bred[warp][8 * g + c] = bsum[c];
        __syncthreads();
        if (t < CH) mine[96 * 96 + t] = alive ? (bred[0][t] + bred[1][t]) + (bred[2][t] + bred[3][t]) : 0.0f;
    }
    bamf::tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) bamf::tc::tmem_dealloc(tbase, 128);
}

/* Column sums of a row-major [nrows][width] array of partial sums, in a
 * fixed order (no atomics: the same bits every run).  A CTA of 32 warps owns
 * 32 consecutive columns (lane = column, coalesced): warp w adds rows w,
 * w + 32, ... into four interleaved accumulators; then warp 0 adds the 32
 * warp sums in order.  The result is valid in warp 0. */
__device__ __forceinline__ float column_sum(const float *__restrict__ part, int nrows, int width, int j,
                                            float (*red)[33])
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f; /* four loads in flight */
    if (j < width) {
        int c = w;
        for (; c + 96 < nrows; c += 128) {
            a0 += part[(size_t)c * width + j];
            a1 += part[(size_t)(c + 32) * width + j];
            a2 += part[(size_t)(c + 64) * width + j];
            a3 += part[(size_t)(c + 96) * width + j];
        }
        for (; c < nrows; c += 32) a0 += part[(size_t)c * width + j];
    }
    red[w][lane] = (a0 + a1) + (a2 + a3);
    __syncthreads();
    float sum = 0.0f;
    if (w == 0)
        for (int k = 0; k < 32; ++k) sum += red[k][lane];
    return sum;
}

/* out[j] += sum over rows of part[row][j], j < width */
__global__ void __launch_bounds__(1024) reduce_rows_kernel(const float *__restrict__ part, int nrows, int width,
                                                           float *__restrict__ out)
{
    __shared__ float red[32][33];
    const int j = blockIdx.x * 32 + (threadIdx.x & 31);
    const float sum = column_sum(part, nrows, width, j, red);
    if (threadIdx.x < 32 && j < width) out[j] += sum;
}

/* dW[co][ci][3 kx + ky] += sum over CTAs of part[cta][(32 kx + co) * 96 +
 * 32 ky + ci], db[c] += sum of part[cta][96 * 96 + c] */
__global__ void __launch_bounds__(1024) dw_reduce_kernel(const float *__restrict__ part, int nparts,
                                                         float *__restrict__ dW, float *__restrict__ db)
{
    __shared__ float red[32][33];
    const int j = blockIdx.x * 32 + (threadIdx.x & 31);
    const float sum = column_sum(part, nparts, DW_PART, j, red);
    if (threadIdx.x < 32 && j < DW_PART) {
        if (j < 96 * 96) {
            const int col = j / 96, row = j - col * 96;
            const int kx = col >> 5, co = col & 31, ky = row >> 5, ci = row & 31;
            dW[(co * CH + ci) * 9 + 3 * kx + ky] += sum;
        } else {
            db[j - 96 * 96] += sum;
        }
    }
}

/* ----------------------------------------------------------------- heads */
/* One CTA (256 threads, thread = pixel) per ROI.  TRAIN: loss, head
 * gradients (row r of `hrows`, HEAD_NPARAM floats per ROI), dz4 = dL/d(pre-
 * activation of conv4).  INFER: the sampler's birth tables and the count
 * logits. */
template <bool TRAIN>
__global__ void __launch_bounds__(256) head_kernel(const bf16 *__restrict__ a4, int n, const float *__restrict__ P,
                                                   const int32_t *__restrict__ n_em, const float *__restrict__ xyi,
                                                   float inv_batch, float *__restrict__ hrows, bf16 *__restrict__ dz4,
                                                   float *__restrict__ loss_buf, const int *__restrict__ step_dev,
                                                   float *__restrict__ cdf, float *__restrict__ sub,
                                                   float *__restrict__ cnt_out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *H = (float *)smem_raw;             /* [256][HS] */
    float *DZ = H + NPX * HS;                 /* [256][17] */
    __shared__ __align__(16) float Wl[NSUB * CH];
    __shared__ float bl[NSUB], Wc[NC * CH], bc[NC];
    __shared__ float red[8], gmean[CH], part[8][CH], zc[NC], dzc[NC], dg[CH];
    __shared__ float ex[BAMF_SYNTH_NMAX], ey[BAMF_SYNTH_NMAX];
    __shared__ float sm_max, sm_sum, loss_loc_sh;
    const int r = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (r >= n) return;
    for (int i = t; i < NSUB * CH; i += 256) Wl[i] = P[O_WL + i];
    for (int i = t; i < NC * CH; i += 256) Wc[i] = P[O_WC + i];
    if (t < NSUB) bl[t] = P[O_BL + t];
    if (t < NC) bc[t] = P[O_BC + t];
    float h[CH];
    {
        const uint4 *src = (const uint4 *)(a4 + ((size_t)r * NPX + t) * CH);
        for (int qd = 0; qd < 4; ++qd) {
            uint4 u = src[qd];
            const bf16 *b = (const bf16 *)&u;
            for (int e = 0; e < 8; ++e) h[qd * 8 + e] = __bfloat162float(b[e]);
        }
    }
#pragma unroll
    for (int q = 0; q < CH / 4; ++q)
        ((float4 *)H)[t * (HS / 4) + q] = make_float4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
    __syncthreads();
    float z[NSUB];
    float mx = -INFINITY;
    for (int s = 0; s < NSUB; ++s) {
        float v = bl[s];
#pragma unroll
        for (int q = 0; q < CH / 4; ++q) {
            const float4 w = ((const float4 *)Wl)[s * (CH / 4) + q];
            v += w.x * h[4 * q];
            v += w.y * h[4 * q + 1];
            v += w.z * h[4 * q + 2];
            v += w.w * h[4 * q + 3];
        }
        z[s] = v;
        mx = fmaxf(mx, v);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) red[warp] = mx;
    /* count head: mean of a4 over pixels */
    {
        int c = t & 31, grp = t >> 5;
        float sacc = 0.0f;
        for (int p = grp; p < NPX; p += 8) sacc += H[p * HS + c];
        part[grp][c] = sacc;
    }
    __syncthreads();
    if (t == 0) {
        float m = red[0];
        for (int k = 1; k < 8; ++k) m = fmaxf(m, red[k]);
        sm_max = m;
    }
    if (t < CH) {
        float sacc = 0.0f;
        for (int k = 0; k < 8; ++k) sacc += part[k][t];
        gmean[t] = sacc * (1.0f / NPX);
    }
    __syncthreads();
    float e[NSUB], se = 0.0f;
    for (int s = 0; s < NSUB; ++s) {
        e[s] = expf(z[s] - sm_max);
        se += e[s];
    }
    float tot = se;
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) red[warp] = tot;
    if (t < NC) {
        float v = bc[t];
        for (int c = 0; c < CH; ++c) v += Wc[t * CH + c] * gmean[c];
        zc[t] = v;
    }
    __syncthreads();
    if (t == 0) {
        float sacc = 0.0f;
        for (int k = 0; k < 8; ++k) sacc += red[k];
        sm_sum = sacc;
    }
    __syncthreads();
    const float inv_sum = 1.0f / sm_sum;
    if (!TRAIN) {
        /* pixel probability, inclusive scan over pixels (thread order = p) */
        float pp = se * inv_sum;
        float incl = pp;
        for (int o = 1; o < 32; o <<= 1) {
            float v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        __syncthreads();
        if (lane == 31) red[warp] = incl;
        __syncthreads();
        float base = 0.0f;
        for (int k = 0; k < warp; ++k) base += red[k];
        cdf[(size_t)r * NPX + t] = base + incl;
        float inv_se = 1.0f / se;
        for (int s = 0; s < NSUB; ++s) sub[((size_t)r * NPX + t) * NSUB + s] = e[s] * inv_se;
        if (cnt_out && t < NC) cnt_out[(size_t)r * NC + t] = zc[t];
        return;
    }
    /* ---- training: targets, loss, gradients */
    const int ntrue = n_em[r];
    if (t < BAMF_SYNTH_NMAX) {
        ex[t] = xyi[((size_t)r * BAMF_SYNTH_NMAX + t) * 3 + 0];
        ey[t] = xyi[((size_t)r * BAMF_SYNTH_NMAX + t) * 3 + 1];
    }
    if (t == 0) loss_loc_sh = 0.0f;
    __syncthreads();
    const int px = t / S, py = t - (t / S) * S;
    float tgt[NSUB];
    for (int s = 0; s < NSUB; ++s) tgt[s] = 0.0f;
    int nin = 0;
    for (int k = 0; k < ntrue; ++k) {
        float X = ex[k], Y = ey[k];
        if (!(X >= 0.0f && X < (float)S && Y >= 0.0f && Y < (float)S)) continue;
        nin++;
        int cx = min((int)X, S - 1), cy = min((int)Y, S - 1);
        if (cx == px && cy == py) {
            int s = min((int)((Y - (float)cy) * 4.0f), 3) + 4 * min((int)((X - (float)cx) * 4.0f), 3);
            tgt[s] += 1.0f;
        }
    }
    const float wloc = nin > 0 ? 1.0f / (float)nin : 0.0f;
    float lloc = 0.0f;
    const float logS = logf(sm_sum) + sm_max;
    for (int s = 0; s < NSUB; ++s) {
        if (tgt[s] > 0.0f) lloc -= tgt[s] * wloc * (z[s] - logS);
        float d = (e[s] * inv_sum - tgt[s] * wloc) * (nin > 0 ? inv_batch : 0.0f);
        DZ[t * (NSUB + 1) + s] = d;
    }
    for (int o = 16; o > 0; o >>= 1) lloc += __shfl_xor_sync(0xffffffffu, lloc, o);
    if (lane == 0) atomicAdd(&loss_loc_sh, lloc);
    if (t == 0) {
        float m = zc[0];
        for (int c = 1; c < NC; ++c) m = fmaxf(m, zc[c]);
        float sacc = 0.0f;
        for (int c = 0; c < NC; ++c) sacc += expf(zc[c] - m);
        int cls = min(ntrue, NC - 1);
        float lcnt = -(zc[cls] - m - logf(sacc));
        for (int c = 0; c < NC; ++c) dzc[c] = (expf(zc[c] - m) / sacc - (c == cls ? 1.0f : 0.0f)) * inv_batch;
        red[0] = lcnt;
    }
    __syncthreads();
    if (t == 0) {
        float l = (loss_loc_sh + red[0]) * inv_batch;
        atomicAdd(&loss_buf[step_dev ? *step_dev : 0], l);
    }
    if (t < CH) {
        float v = 0.0f;
        for (int c = 0; c < NC; ++c) v += Wc[c * CH + t] * dzc[c];
        dg[t] = v * (1.0f / NPX);
    }
    __syncthreads();
    /* dz4 of this pixel */
    {
        float dzr[NSUB];
#pragma unroll
        for (int k = 0; k < NSUB; ++k) dzr[k] = DZ[t * (NSUB + 1) + k];
        __align__(16) bf16 o[CH];
#pragma unroll
        for (int q = 0; q < CH / 4; ++q) {
            float v0 = dg[4 * q], v1 = dg[4 * q + 1], v2 = dg[4 * q + 2], v3 = dg[4 * q + 3];
#pragma unroll
            for (int k = 0; k < NSUB; ++k) {
                const float4 w = ((const float4 *)Wl)[k * (CH / 4) + q];
                v0 += dzr[k] * w.x;
                v1 += dzr[k] * w.y;
                v2 += dzr[k] * w.z;
                v3 += dzr[k] * w.w;
            }
            o[4 * q] = __float2bfloat16_rn(h[4 * q] > 0.0f ? v0 : 0.0f);
            o[4 * q + 1] = __float2bfloat16_rn(h[4 * q + 1] > 0.0f ? v1 : 0.0f);
            o[4 * q + 2] = __float2bfloat16_rn(h[4 * q + 2] > 0.0f ? v2 : 0.0f);
            o[4 * q + 3] = __float2bfloat16_rn(h[4 * q + 3] > 0.0f ? v3 : 0.0f);
        }
        uint4 *dst = (uint4 *)(dz4 + ((size_t)r * NPX + t) * CH);
        const uint4 *src = (const uint4 *)o;
        for (int qd = 0; qd < 4; ++qd) dst[qd] = src[qd];
    }
    /* head parameter gradients of this ROI, in the parameter order from O_WL
     * (WL, BL, WC, BC), into its row of `hrows` (one row per ROI; reduce_rows_kernel
     * adds the rows).  dWL[s][c] = sum over pixels of DZ[p][s] H[p][c] and
     * dBL[s] = sum of DZ[p][s]: thread t owns the 2 x 4 block (s0, c0) of
     * tile t & 63 over the pixel quarter t >> 6; the four quarters are added
     * through shared memory (over H, once every thread has read it). */
    {
        const int tile = t & 63, quarter = t >> 6;
        const int s0 = 2 * (tile >> 3), c0 = 4 * (tile & 7);
        float g0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, g1[4] = {0.0f, 0.0f, 0.0f, 0.0f}, gb0 = 0.0f, gb1 = 0.0f;
#pragma unroll 4
        for (int p = 64 * quarter; p < 64 * quarter + 64; ++p) {
            const float4 hv = ((const float4 *)H)[p * (HS / 4) + (c0 >> 2)];
            const float d0 = DZ[p * (NSUB + 1) + s0], d1 = DZ[p * (NSUB + 1) + s0 + 1];
            g0[0] += d0 * hv.x;
            g0[1] += d0 * hv.y;
            g0[2] += d0 * hv.z;
            g0[3] += d0 * hv.w;
            g1[0] += d1 * hv.x;
            g1[1] += d1 * hv.y;
            g1[2] += d1 * hv.z;
            g1[3] += d1 * hv.w;
            gb0 += d0;
            gb1 += d1;
        }
        __syncthreads();
        constexpr int QW = NSUB * CH + NSUB; /* one quarter's WL and BL sums */
        float *red = H + quarter * QW;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            red[s0 * CH + c0 + k] = g0[k];
            red[(s0 + 1) * CH + c0 + k] = g1[k];
        }
        if ((tile & 7) == 0) {
            red[NSUB * CH + s0] = gb0;
            red[NSUB * CH + s0 + 1] = gb1;
        }
        __syncthreads();
        float *row = hrows + (size_t)r * HEAD_NPARAM;
        for (int o = t; o < QW; o += 256) row[o] = (H[o] + H[QW + o]) + (H[2 * QW + o] + H[3 * QW + o]);
    }
    for (int o = t; o < NC * CH; o += 256) row_wc(hrows, r)[o] = dzc[o / CH] * gmean[o - (o / CH) * CH];
    if (t < NC) row_wc(hrows, r)[NC * CH + t] = dzc[t];
}

/* --------------------------------------------------------- start states */
/* A chain start per ROI from the network: n0 = argmax of the count logits
 * (at most max_n), positions = the n0 most probable sub-cells, greedily,
 * each suppressing the cells within 1 px of it; intensity `intensity`.
 * One CTA (256 threads, thread = pixel) per ROI. */
__global__ void __launch_bounds__(256) init_kernel(const float *__restrict__ cdf, const float *__restrict__ sub,
                                                   const float *__restrict__ cnt, int n, float intensity,
                                                   int max_n, int32_t *__restrict__ init_n,
                                                   float *__restrict__ init_ixy)
{
    __shared__ float bv[8];
    __shared__ int bi[8];
    __shared__ int win;
    const int r = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (r >= n) return;
    int n0 = 0;
    {
        const float *c = cnt + (size_t)r * NC;
        float m = c[0];
        for (int k = 1; k < NC; ++k)
            if (c[k] > m) {
                m = c[k];
                n0 = k;
            }
        n0 = min(n0, max_n);
    }
    const float pp = cdf[(size_t)r * NPX + t] - (t > 0 ? cdf[(size_t)r * NPX + t - 1] : 0.0f);
    float pr[NSUB];
    for (int s = 0; s < NSUB; ++s) pr[s] = pp * sub[((size_t)r * NPX + t) * NSUB + s];
    const int px = t / S, py = t - (t / S) * S;
    float *ixy = init_ixy + (size_t)r * 3 * BAMF_NMAX;
    for (int k = 0; k < n0; ++k) {
        float v = -1.0f;
        int idx = 0;
        for (int s = 0; s < NSUB; ++s)
            if (pr[s] > v) {
                v = pr[s];
                idx = t * NSUB + s;
            }
        for (int o = 16; o > 0; o >>= 1) {
            float ov = __shfl_xor_sync(0xffffffffu, v, o);
            int oi = __shfl_xor_sync(0xffffffffu, idx, o);
            if (ov > v || (ov == v && oi < idx)) {
                v = ov;
                idx = oi;
            }
        }
        if (lane == 0) {
            bv[warp] = v;
            bi[warp] = idx;
        }
        __syncthreads();
        if (t == 0) {
            float m = bv[0];
            int w = bi[0];
            for (int q = 1; q < 8; ++q)
                if (bv[q] > m || (bv[q] == m && bi[q] < w)) {
                    m = bv[q];
                    w = bi[q];
                }
            win = w;
        }
        __syncthreads();
        const int wp = win / NSUB, ws = win - (win / NSUB) * NSUB;
        const float wx = (float)(wp / S) + ((float)(ws >> 2) + 0.5f) * 0.25f;
        const float wy = (float)(wp - (wp / S) * S) + ((float)(ws & 3) + 0.5f) * 0.25f;
        if (t == 0) {
            ixy[k] = intensity;
            ixy[BAMF_NMAX + k] = wx;
            ixy[2 * BAMF_NMAX + k] = wy;
        }
        for (int s = 0; s < NSUB; ++s) {
            float cx = (float)px + ((float)(s >> 2) + 0.5f) * 0.25f, cy = (float)py + ((float)(s & 3) + 0.5f) * 0.25f;
            if ((cx - wx) * (cx - wx) + (cy - wy) * (cy - wy) < 1.0f) pr[s] = 0.0f;
        }
        __syncthreads();
    }
    if (t == 0) init_n[r] = n0;
}

/* ------------------------------------------------------------------ Adam */
__global__ void adam_kernel(float *__restrict__ P, float *__restrict__ G, float *__restrict__ m,
                            float *__restrict__ v, const int *__restrict__ step_dev, int steps_total, float lr0)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    int step = *step_dev;
    float frac = steps_total > 1 ? (float)step / (float)(steps_total - 1) : 0.0f;
    float lr = lr0 * (1.0f - 0.9f * fminf(frac, 1.0f));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float g = G[i];
    float mi = b1 * m[i] + (1.0f - b1) * g;
    float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float t = (float)(step + 1);
    float mh = mi / (1.0f - powf(b1, t));
    float vh = vi / (1.0f - powf(b2, t));
    P[i] -= lr * mh / (sqrtf(vh) + eps);
    G[i] = 0.0f;
}

__global__ void step_inc_kernel(int *step_dev) { *step_dev += 1; }

/* Training batch `step` from caller-provided examples: ROI b of the batch is
 * example (step * batch + b) mod n_examples; counts clipped to the target
 * capacity.  One CTA of NPX threads per ROI. */
__global__ void gather_examples_kernel(const float *__restrict__ data, const int32_t *__restrict__ n_em,
                                       const float *__restrict__ xyi, int n_examples, const int *step_dev,
                                       int batch, float *__restrict__ gdata, int32_t *__restrict__ gn,
                                       float *__restrict__ gxyi)
{
    const int b = blockIdx.x, t = threadIdx.x;
    const int64_t k = ((int64_t)(*step_dev) * batch + b) % n_examples;
    gdata[(size_t)b * NPX + t] = data[(size_t)k * NPX + t];
    if (t == 0) gn[b] = min(max(n_em[k], 0), BAMF_SYNTH_NMAX);
    if (t < BAMF_SYNTH_NMAX * 3) gxyi[(size_t)b * BAMF_SYNTH_NMAX * 3 + t] = xyi[(size_t)k * BAMF_SYNTH_NMAX * 3 + t];
}

}  // namespace

/* ================================================================ host */
struct bamf_cnn {
    float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;
    bf16 *Wf = nullptr, *Wb = nullptr;
    /* batch buffers (MAX_BATCH) */
    float *x0 = nullptr;
    bf16 *a[4] = {nullptr, nullptr, nullptr, nullptr};
    bf16 *dzA = nullptr, *dzB = nullptr;
    float *gdata = nullptr, *gxyi = nullptr;
    int32_t *gn = nullptr;
    int *step = nullptr;
    int *tc_status = nullptr; /* set by a convolution whose tensor-core wait timed out */
    float *dwpart = nullptr;  /* per-CTA partial weight gradients, 2 CTAs per SM */
    float *hpart = nullptr;   /* per-ROI head gradients (MAX_BATCH rows) */
    float *c1part = nullptr;  /* per-CTA conv1 gradients, 4 CTAs per SM */
    float *loss = nullptr;
    int loss_cap = 0;
    int sms = 1;
    bool packed = false;
};

namespace {

std::mutex g_attr_mutex;
bool g_attr_done = false;

const size_t SMEM_HEAD = (size_t)(NPX * HS + NPX * (NSUB + 1)) * sizeof(float);

cudaError_t set_attrs()
{
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    if (g_attr_done) return cudaSuccess;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(conv_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC)))
        return e;
    if ((e = cudaFuncSetAttribute(conv_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC)))
        return e;
    if ((e = cudaFuncSetAttribute(conv_dw_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_DW)))
        return e;
    if ((e = cudaFuncSetAttribute(head_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_HEAD)))
        return e;
    if ((e = cudaFuncSetAttribute(head_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_HEAD)))
        return e;
    g_attr_done = true;
    return cudaSuccess;
}

#define CK(x)                                                                                                    \
    do {                                                                                                         \
        cudaError_t e_ = (x);                                                                                    \
        if (e_ != cudaSuccess) {                                                                                 \
            cudaGetLastError();                                                                                  \
            return BAMF_ERR_CUDA;                                                                                \
        }                                                                                                        \
    } while (0)

int grid_for(int n, int per_sm, int sms) { return std::max(1, std::min(n, per_sm * sms)); }

/* forward of a batch of n <= capacity ROIs from data, activations kept */
bamf_status forward(bamf_cnn *net, const float *data, int n, cudaStream_t s)
{
    conv1_fwd_kernel<<<n, 256, 0, s>>>(data, n, net->P, net->x0, net->a[0]);
    for (int l = 0; l < 3; ++l)
        conv_tc_kernel<0><<<grid_for(n, 3, net->sms), 128, SMEM_TC, s>>>(net->a[l], net->Wf + l * PKT,
                                                                         net->P + O_B[l], nullptr, net->a[l + 1], n,
                                                                         net->tc_status);
    CK(cudaGetLastError());
    return BAMF_OK;
}

/* loss and gradients (accumulated into G) of the batch whose forward ran */
bamf_status backward(bamf_cnn *net, const int32_t *n_em, const float *xyi, int n, float inv_batch, cudaStream_t s)
{
    head_kernel<true><<<n, 256, SMEM_HEAD, s>>>(net->a[3], n, net->P, n_em, xyi, inv_batch, net->hpart, net->dzA,
                                                net->loss, net->step, nullptr, nullptr, nullptr);
    bf16 *dz = net->dzA, *dzn = net->dzB;
    for (int l = 2; l >= 0; --l) {
        /* layer l+2: input a[l], output a[l+1]; dz = dL/dz_{l+2} */
        const int gdw = grid_for(n, 2, net->sms);
        conv_dw_tc_kernel<<<gdw, 128, SMEM_DW, s>>>(net->a[l], dz, n, net->dwpart, net->tc_status);
        dw_reduce_kernel<<<(DW_PART + 31) / 32, 1024, 0, s>>>(net->dwpart, gdw, net->G + O_W[l], net->G + O_B[l]);
        conv_tc_kernel<1><<<grid_for(n, 3, net->sms), 128, SMEM_TC, s>>>(dz, net->Wb + l * PKT, nullptr,
                                                                         net->a[l], dzn, n, net->tc_status);
        bf16 *tmp = dz;
        dz = dzn;
        dzn = tmp;
    }
    reduce_rows_kernel<<<(HEAD_NPARAM + 31) / 32, 1024, 0, s>>>(net->hpart, n, HEAD_NPARAM, net->G + O_WL);
    const int g1 = grid_for(n, 4, net->sms);
    conv1_bwd_kernel<<<g1, 256, 0, s>>>(net->x0, dz, n, net->c1part);
    reduce_rows_kernel<<<(C1_NPARAM + 31) / 32, 1024, 0, s>>>(net->c1part, g1, C1_NPARAM, net->G + O_W1);
    CK(cudaGetLastError());
    return BAMF_OK;
}

bamf_status pack(bamf_cnn *net, cudaStream_t s)
{
    pack_kernel<<<(3 * 9 * CH * CH + 255) / 256, 256, 0, s>>>(net->P, net->Wf, net->Wb);
    CK(cudaGetLastError());
    return BAMF_OK;
}

}  // namespace

extern "C" bamf_status bamf_synth_generate(const bamf_synth_params *sp, uint32_t seed, uint64_t first, int n,
                                           float *data, int32_t *n_em, float *xyi, void *stream)
{
    if (!sp || n < 0 || (n > 0 && (!data || !n_em || !xyi))) return BAMF_ERR_INVALID_ARG;
    if (!(sp->sigma > 0.0f) || !(sp->mean_n >= 0.0f) || !(sp->i_median > 0.0f) || !(sp->bg >= 0.0f))
        return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    synth_kernel<<<n, 256, 0, (cudaStream_t)stream>>>(*sp, seed, first, nullptr, 0, n, data, n_em, xyi);
    CK(cudaGetLastError());
    return BAMF_OK;
}

extern "C" void bamf_cnn_destroy(bamf_cnn *net)
{
    if (!net) return;
    void *ps[] = {net->P, net->G, net->M, net->V, net->Wf, net->Wb, net->x0, net->a[0], net->a[1], net->a[2],
                  net->a[3], net->dzA, net->dzB, net->gdata, net->gxyi, net->gn, net->step, net->loss,
                  net->tc_status, net->dwpart, net->hpart, net->c1part};
    for (void *p : ps)
        if (p) cudaFree(p);
    delete net;
}

extern "C" bamf_status bamf_cnn_create(bamf_cnn **out, uint32_t seed)
{
    if (!out) return BAMF_ERR_INVALID_ARG;
    *out = nullptr;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    if (set_attrs() != cudaSuccess) return BAMF_ERR_CUDA;
    bamf_cnn *net = new bamf_cnn();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&net->sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t B = MAX_BATCH;
    bool ok = cudaMalloc(&net->P, NPARAM * 4) == cudaSuccess && cudaMalloc(&net->G, NPARAM * 4) == cudaSuccess &&
              cudaMalloc(&net->M, NPARAM * 4) == cudaSuccess && cudaMalloc(&net->V, NPARAM * 4) == cudaSuccess &&
              cudaMalloc(&net->Wf, 3 * PKT * 2) == cudaSuccess && cudaMalloc(&net->Wb, 3 * PKT * 2) == cudaSuccess &&
              cudaMalloc(&net->tc_status, sizeof(int)) == cudaSuccess &&
              cudaMalloc(&net->dwpart, (size_t)2 * net->sms * DW_PART * 4) == cudaSuccess &&
              cudaMalloc(&net->hpart, B * HEAD_NPARAM * 4) == cudaSuccess &&
              cudaMalloc(&net->c1part, (size_t)4 * net->sms * C1_NPARAM * 4) == cudaSuccess &&
              cudaMalloc(&net->x0, B * NPX * 4) == cudaSuccess && cudaMalloc(&net->dzA, B * NPX * CH * 2) == cudaSuccess &&
              cudaMalloc(&net->dzB, B * NPX * CH * 2) == cudaSuccess &&
              cudaMalloc(&net->gdata, B * NPX * 4) == cudaSuccess &&
              cudaMalloc(&net->gxyi, B * BAMF_SYNTH_NMAX * 3 * 4) == cudaSuccess &&
              cudaMalloc(&net->gn, B * 4) == cudaSuccess && cudaMalloc(&net->step, sizeof(int)) == cudaSuccess;
    for (int l = 0; l < 4 && ok; ++l) ok = cudaMalloc(&net->a[l], B * NPX * CH * 2) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        bamf_cnn_destroy(net);
        return BAMF_ERR_CUDA;
    }
    /* He initialisation from a Philox stream (Box-Muller), zero biases */
    std::vector<float> h(NPARAM, 0.0f);
    uint32_t ctr = 0;
    auto normal = [&]() {
        bamf_philox_block b = bamf_philox4x32_10(ctr++, 0u, 0u, 0u, seed, 0x2545F491u);
        double u1 = ((double)(b.v[0] >> 8) + 0.5) / 16777216.0, u2 = ((double)(b.v[1] >> 8) + 0.5) / 16777216.0;
        return (float)(std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2));
    };
    auto fill = [&](int off, int count, int fan_in) {
        float sd = std::sqrt(2.0f / (float)fan_in);
        for (int i = 0; i < count; ++i) h[off + i] = sd * normal();
    };
    fill(O_W1, 288, 9);
    fill(O_W2, 9216, 288);
    fill(O_W3, 9216, 288);
    fill(O_W4, 9216, 288);
    fill(O_WL, 512, 32);
    fill(O_WC, 352, 32);
    bool ok2 = cudaMemcpy(net->P, h.data(), NPARAM * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
               cudaMemset(net->G, 0, NPARAM * 4) == cudaSuccess && cudaMemset(net->M, 0, NPARAM * 4) == cudaSuccess &&
               cudaMemset(net->V, 0, NPARAM * 4) == cudaSuccess && cudaMemset(net->step, 0, sizeof(int)) == cudaSuccess &&
               cudaMemset(net->tc_status, 0, sizeof(int)) == cudaSuccess;
    if (!ok2 || pack(net, nullptr) != BAMF_OK || cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        bamf_cnn_destroy(net);
        return BAMF_ERR_CUDA;
    }
    *out = net;
    return BAMF_OK;
}

extern "C" bamf_status bamf_cnn_get_params(bamf_cnn *net, float *params)
{
    if (!net || !params) return BAMF_ERR_INVALID_ARG;
    CK(cudaMemcpy(params, net->P, NPARAM * 4, cudaMemcpyDeviceToHost));
    return BAMF_OK;
}

extern "C" bamf_status bamf_cnn_set_params(bamf_cnn *net, const float *params)
{
    if (!net || !params) return BAMF_ERR_INVALID_ARG;
    CK(cudaMemcpy(net->P, params, NPARAM * 4, cudaMemcpyHostToDevice));
    bamf_status r = pack(net, nullptr);
    if (r) return r;
    CK(cudaDeviceSynchronize());
    return BAMF_OK;
}

/* after a synchronisation: a convolution whose tensor-core completion wait
 * ran out left garbage outputs; report it */
static bamf_status check_tc(bamf_cnn *net)
{
    int st = 0;
    CK(cudaMemcpy(&st, net->tc_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        cudaMemset(net->tc_status, 0, sizeof(int));
        return BAMF_ERR_CUDA;
    }
    return BAMF_OK;
}

static bamf_status ensure_loss(bamf_cnn *net, int cap)
{
    if (net->loss_cap >= cap) return BAMF_OK;
    if (net->loss) cudaFree(net->loss);
    net->loss = nullptr;
    net->loss_cap = 0;
    CK(cudaMalloc(&net->loss, (size_t)cap * sizeof(float)));
    net->loss_cap = cap;
    return BAMF_OK;
}

extern "C" bamf_status bamf_cnn_loss_grad(bamf_cnn *net, const float *data, const int32_t *n_em, const float *xyi,
                                          int n, float *loss, float *grad)
{
    if (!net || !data || !n_em || !xyi || n < 1 || n > MAX_BATCH) return BAMF_ERR_INVALID_ARG;
    bamf_status r;
    if ((r = ensure_loss(net, 1))) return r;
    int saved = 0;
    CK(cudaMemcpy(&saved, net->step, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemset(net->step, 0, sizeof(int)));
    CK(cudaMemset(net->loss, 0, sizeof(float)));
    CK(cudaMemset(net->G, 0, NPARAM * 4));
    if ((r = forward(net, data, n, nullptr))) return r;
    if ((r = backward(net, n_em, xyi, n, 1.0f / (float)n, nullptr))) return r;
    CK(cudaDeviceSynchronize());
    if ((r = check_tc(net))) return r;
    if (loss) CK(cudaMemcpy(loss, net->loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (grad) CK(cudaMemcpy(grad, net->G, NPARAM * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemset(net->G, 0, NPARAM * 4));
    CK(cudaMemcpy(net->step, &saved, sizeof(int), cudaMemcpyHostToDevice));
    return BAMF_OK;
}

/* `steps` Adam steps, each one replay of a CUDA graph of: produce(s) (the
 * step's batch into gdata / gn / gxyi), forward, backward, Adam, weight
 * packing, step counter.  Optimiser state starts from zero. */
template <typename Produce>
static bamf_status train_graph(bamf_cnn *net, int steps, int batch, float lr, float *loss_trace, Produce produce)
{
    bamf_status r;
    if ((r = ensure_loss(net, steps))) return r;
    cudaStream_t s;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bamf_status res = BAMF_OK;
    do {
        if (cudaMemsetAsync(net->step, 0, sizeof(int), s) != cudaSuccess ||
            cudaMemsetAsync(net->loss, 0, (size_t)steps * sizeof(float), s) != cudaSuccess ||
            cudaMemsetAsync(net->G, 0, NPARAM * 4, s) != cudaSuccess ||
            cudaMemsetAsync(net->M, 0, NPARAM * 4, s) != cudaSuccess ||
            cudaMemsetAsync(net->V, 0, NPARAM * 4, s) != cudaSuccess) {
            res = BAMF_ERR_CUDA;
            break;
        }
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            res = BAMF_ERR_CUDA;
            break;
        }
        produce(s);
        bamf_status r1 = forward(net, net->gdata, batch, s);
        bamf_status r2 = r1 ? r1 : backward(net, net->gn, net->gxyi, batch, 1.0f / (float)batch, s);
        adam_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(net->P, net->G, net->M, net->V, net->step, steps, lr);
        pack_kernel<<<(3 * 9 * CH * CH + 255) / 256, 256, 0, s>>>(net->P, net->Wf, net->Wb);
        step_inc_kernel<<<1, 1, 0, s>>>(net->step);
        cudaError_t ec = cudaStreamEndCapture(s, &graph);
        if (r2 || ec != cudaSuccess) {
            res = r2 ? r2 : BAMF_ERR_CUDA;
            break;
        }
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            res = BAMF_ERR_CUDA;
            break;
        }
        for (int i = 0; i < steps; ++i)
            if (cudaGraphLaunch(exec, s) != cudaSuccess) {
                res = BAMF_ERR_CUDA;
                break;
            }
        if (res) break;
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            res = BAMF_ERR_CUDA;
            break;
        }
        if ((res = check_tc(net))) break;
        if (loss_trace &&
            cudaMemcpy(loss_trace, net->loss, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
            res = BAMF_ERR_CUDA;
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(s);
    if (res) cudaGetLastError();
    return res;
}

extern "C" bamf_status bamf_cnn_train(bamf_cnn *net, const bamf_synth_params *sp, int steps, int batch, float lr,
                                      uint32_t data_seed, float *loss_trace)
{
    if (!net || !sp || steps < 0 || batch < 1 || batch > MAX_BATCH || !(lr > 0.0f)) return BAMF_ERR_INVALID_ARG;
    if (steps == 0) return BAMF_OK;
    const bamf_synth_params spv = *sp;
    return train_graph(net, steps, batch, lr, loss_trace, [&](cudaStream_t s) {
        synth_kernel<<<batch, 256, 0, s>>>(spv, data_seed, 0, net->step, batch, batch, net->gdata, net->gn,
                                           net->gxyi);
    });
}

extern "C" bamf_status bamf_cnn_train_examples(bamf_cnn *net, const float *data, const int32_t *n_em,
                                               const float *xyi, int n_examples, int steps, int batch, float lr,
                                               float *loss_trace)
{
    if (!net || !data || !n_em || !xyi || n_examples < 1 || steps < 0 || batch < 1 || batch > MAX_BATCH ||
        !(lr > 0.0f))
        return BAMF_ERR_INVALID_ARG;
    if (steps == 0) return BAMF_OK;
    return train_graph(net, steps, batch, lr, loss_trace, [&](cudaStream_t s) {
        gather_examples_kernel<<<batch, NPX, 0, s>>>(data, n_em, xyi, n_examples, net->step, batch, net->gdata,
                                                     net->gn, net->gxyi);
    });
}

extern "C" bamf_status bamf_cnn_init_states(const float *cdf, const float *sub, const float *count_logits, int n,
                                            float intensity, int max_n, int32_t *init_n, float *init_ixy,
                                            void *stream)
{
    if (n < 0 || max_n < 0 || max_n > BAMF_NMAX) return BAMF_ERR_INVALID_ARG;
    if (n > 0 && (!cdf || !sub || !count_logits || !init_n || !init_ixy)) return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    init_kernel<<<n, 256, 0, (cudaStream_t)stream>>>(cdf, sub, count_logits, n, intensity, max_n, init_n, init_ixy);
    CK(cudaGetLastError());
    return BAMF_OK;
}

extern "C" bamf_status bamf_cnn_infer(bamf_cnn *net, const float *data, int n, float *cdf, float *sub,
                                      float *count_logits, void *stream)
{
    if (!net || n < 0 || (n > 0 && (!data || !cdf || !sub))) return BAMF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    for (int b0 = 0; b0 < n; b0 += MAX_BATCH) {
        int m = std::min(MAX_BATCH, n - b0);
        bamf_status r = forward(net, data + (size_t)b0 * NPX, m, s);
        if (r) return r;
        head_kernel<false><<<m, 256, SMEM_HEAD, s>>>(net->a[3], m, net->P, nullptr, nullptr, 0.0f, nullptr, nullptr,
                                                     nullptr, nullptr, cdf + (size_t)b0 * NPX,
                                                     sub + (size_t)b0 * NPX * NSUB,
                                                     count_logits ? count_logits + (size_t)b0 * NC : nullptr);
        CK(cudaGetLastError());
    }
    return BAMF_OK;
}
