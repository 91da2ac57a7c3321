/*
 * sampler_kernel.cuh - the batched RJMCMC sampler (cRJMCMC's algorithm,
 * source/c/LibRJMCMC.cpp) as a persistent CUDA kernel for sm_103a.
 *
 * Layout of the work:
 *   - one warp runs one ROI chain from burn-in to the last trial, then pulls
 *     the next ROI id from a device work queue (atomic counter);
 *   - lane j holds emitter slot j (I, X, Y, Signal) of the current state A
 *     and of the proposed state T in registers (BAMF_NMAX = 32 slots), so
 *     emitter edits are register moves and neighbour searches are ballots;
 *   - the ROI pixels D, the current model M, the proposed model Mt and the
 *     per-pixel work buffer live in shared memory; pixel p = y + x*Ysize is
 *     handled by lane p mod 32;
 *   - the scalar move logic (proposal, priors, Hastings ratio, accept) runs
 *     warp-uniformly: every lane evaluates it on the same values, so no
 *     broadcasts are needed and the warp never diverges there;
 *   - uniforms come from the chain's Philox stream (include/bamf_philox.h):
 *     each lane generates one 4-word block, 32 blocks = 128 uniforms per
 *     refill, and a draw is one shuffle.
 *
 * Two instantiations (template parameter EXACT):
 *   EXACT = true  (sampler_exact.cu, built with -fmad=false): the reference's
 *     float operation order, parity erf/log/exp, full model rebuild per
 *     proposal and serial pixel sums, so the chain is the reference chain
 *     bit for bit given the same uniforms.
 *   EXACT = false (sampler_fast.cu): hardware math, incremental model
 *     updates (only changed emitters' stencils are evaluated), cached
 *     log-model and warp-tree reductions; same moves and acceptance rule.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bamf.h"
#include "bamf_parity_math.h"
#include "bamf_philox.h"
#include "sampler_common.h"

namespace bamf {

#define BAMF_FULL 0xffffffffu

/* counter slots, in bamf_counters order */
enum {
    C_N_jump, C_N_split, C_N_merge, C_N_birth, C_N_death,
    C_A_jump, C_A_split, C_A_merge, C_A_birth, C_A_death,
    C_N_jumpFg, C_N_splitFg, C_N_mergeFg, C_N_birthFg, C_N_deathFg,
    C_A_jumpFg, C_A_splitFg, C_A_mergeFg, C_A_birthFg, C_A_deathFg,
    C_N_jumpBg, C_N_splitBg, C_N_mergeBg, C_N_birthBg, C_N_deathBg,
    C_A_jumpBg, C_A_splitBg, C_A_mergeBg, C_A_birthBg, C_A_deathBg,
    C_COUNT
};

template <bool EXACT>
struct SMath;

template <>
struct SMath<true> {
    static __device__ __forceinline__ float erf_(float x) { return bamf_pm_erff(x); }
    static __device__ __forceinline__ float log_(float x) { return bamf_pm_logf(x); }
    static __device__ __forceinline__ float exp_(float x) { return bamf_pm_expf(x); }
    static __device__ __forceinline__ float powf_(float x, float y) { return bamf_pm_powf(x, y); }
};

template <>
struct SMath<false> {
    static __device__ __forceinline__ float erf_(float x) { return erff(x); }
    static __device__ __forceinline__ float log_(float x) { return __logf(x); }
    static __device__ __forceinline__ float exp_(float x) { return __expf(x); }
    static __device__ __forceinline__ float powf_(float x, float y) { return powf(x, y); }
};

/* Per-warp shared-memory carve-out, in floats.  Exact: data D, model M,
 * proposal model Mt, per-pixel work E, sCMOS, proposal stencils NX/NY.
 * Fast: D, M, Mt and the compact stencil rows SXo/SYo (old, of A) and
 * SXn/SYn (new, of T); log2 M is recomputed in each likelihood pass (the
 * SFU has room; the smaller carve-out keeps 3 CTAs of 8 chains resident
 * up to 24x24 ROIs); sCMOS is read from global memory at model rebuilds
 * only.  Both: counters and the neighbour pick list. */
/* Fast mode keeps stencil rows only for the emitters a proposal changes:
 * up to FAST_ROWS old rows (A) and FAST_ROWS new rows (T); larger proposals
 * (rare: a jump of a cluster of more than 4 emitters) and periodic rebuilds
 * stream the model one emitter at a time. */
#define FAST_ROWS 4
__host__ __device__ inline int warp_smem_floats(int side_max, bool exact)
{
    int npix = side_max * side_max, nxs = BAMF_NMAX * side_max;
    return exact ? 5 * npix + 4 * nxs + C_COUNT + BAMF_NMAX + 2 /* D M Mt E sCMOS, NX NY of A and of T */
                 : 3 * npix + 4 * FAST_ROWS * side_max + C_COUNT + BAMF_NMAX + 2; /* D M Mt SXo SYo SXn SYn */
}

/* double helpers that nvcc may not contract */
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

/* Out-of-line helpers.  They are called from many places of the chain loop
 * but run rarely per jump; keeping one copy of each keeps the loop's code
 * small enough for the instruction cache (a fully inlined loop spent most
 * of its cycles waiting on instruction fetch). */

/* One Philox4x32-10 block of a chain's stream (include/bamf_philox.h). */
static __device__ __noinline__ uint4 philox_block(uint32_t ctr, uint32_t seed, uint32_t chain)
{
    bamf_philox_block b = bamf_philox4x32_10(ctr, 0u, 0u, 0u, seed, chain);
    return make_uint4(b.v[0], b.v[1], b.v[2], b.v[3]);
}

/* Stat::findPDF (source/c/LibRJMCMC.cpp:219-246): linear interpolation of
 * the pdf at I, 0 outside (0, x[L-1]).  The grid is x[i] = x[i-1] + DX, so
 * the first node strictly above I (what the reference's linear scan finds)
 * is reached from the guess I / DX in a step or two. */
static __device__ __noinline__ float stat_pdf(const float *__restrict__ x, const float *__restrict__ pdf, int L,
                                       float I)
{
    float xl = __ldg(&x[L - 1]);
    if (I >= xl || I <= 0.0f || I != I) return 0.0f;
    float x1 = __ldg(&x[1]);
    int j = min(max((int)(I / x1) + 1, 1), L - 1);
    float xj = __ldg(&x[j]), xj1 = __ldg(&x[j - 1]);
    while (j > 1 && xj1 > I) {
        --j;
        xj = xj1;
        xj1 = __ldg(&x[j - 1]);
    }
    while (j < L - 1 && !(xj > I)) {
        ++j;
        xj1 = xj;
        xj = __ldg(&x[j]);
    }
    return (__ldg(&pdf[j]) * (I - xj1) + __ldg(&pdf[j - 1]) * (xj - I)) / (x1 - __ldg(&x[0]));
}

/* Fast-arithmetic findPDF: the grid is uniform (x[i] = i DX up to float
 * rounding), so the interval of I is found by one multiply and its two
 * nodes are loaded together with the grid's end - one memory round trip
 * instead of a dependent walk.  Same linear interpolation, 0 outside
 * (0, x[L-1]). */
static __device__ __noinline__ float stat_pdf_fast(const float *__restrict__ x, const float *__restrict__ pdf, int L,
                                                   float inv_dx, float I)
{
    if (L < 2) return 0.0f;
    float u = fminf(fmaxf(I * inv_dx, 0.0f), (float)(L - 1)); /* NaN -> 0 */
    int j = min((int)u + 1, L - 1);
    float xl = __ldg(&x[L - 1]);
    float p1 = __ldg(&pdf[j]), p0 = __ldg(&pdf[j - 1]);
    float w = u - (float)(j - 1);
    float v = p1 * w + p0 * (1.0f - w);
    return (I >= xl || I <= 0.0f || I != I) ? 0.0f : v;
}

/* Fast-arithmetic genRand: the same first unique-CDF node above R, found by
 * a 32-way search (each lane tests one candidate, a ballot keeps the
 * bracket: two or three rounds of loads instead of a dependent binary
 * search), then the same interpolation.  Call with the whole warp. */
static __device__ __noinline__ float stat_rand_warp(const float *__restrict__ ux, const float *__restrict__ uc,
                                                    int nu, float R, int lane)
{
    if (R <= 0.0f) return 0.0f;
    if (R >= 1.0f) return __ldg(&ux[nu - 1]);
    if (nu < 2) return 0.0f;
    int lo = 0, hi = nu - 1; /* uc[lo] <= R < uc[hi] */
    while (hi - lo > 1) {
        int step = (hi - lo + 31) >> 5;
        int k = lo + (lane + 1) * step;
        bool above = k >= hi || __ldg(&uc[k]) > R;
        uint32_t m = __ballot_sync(0xffffffffu, above);
        int f = __ffs(m) - 1;
        int nlo = f == 0 ? lo : lo + f * step;
        hi = min(lo + (f + 1) * step, hi);
        lo = nlo;
    }
    float uc1 = __ldg(&uc[hi]), uc0 = __ldg(&uc[hi - 1]);
    return (__ldg(&ux[hi - 1]) * (uc1 - R) + __ldg(&ux[hi]) * (R - uc0)) / (uc1 - uc0);
}

/* Stat::genRand (:248-282) given its uniform R: first unique-CDF node above R
 * by binary search (the CDF is strictly increasing), then interpolation. */
static __device__ __noinline__ float stat_rand(const float *__restrict__ ux, const float *__restrict__ uc, int nu,
                                        float R)
{
    if (R <= 0.0f) return 0.0f;
    if (R >= 1.0f) return __ldg(&ux[nu - 1]);
    if (nu < 2) return 0.0f;
    int lo = 0, hi = nu - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(&uc[mid]) > R) hi = mid; else lo = mid;
    }
    float uc1 = __ldg(&uc[hi]), uc0 = __ldg(&uc[hi - 1]);
    return (__ldg(&ux[hi - 1]) * (uc1 - R) + __ldg(&ux[hi]) * (R - uc0)) / (uc1 - uc0);
}

/* Fast-mode Irwin-Hall draw: lanes 0..11 fetch uniforms idx..idx+11 of the
 * warp's buffered Philox blocks (lane l holds block base+l in r0..r3) and
 * add them in a butterfly.  Call with the whole warp and the 12 draws inside
 * the buffer. */
static __device__ __noinline__ float irwin_hall12(uint32_t idx, uint32_t base, uint32_t r0, uint32_t r1,
                                           uint32_t r2, uint32_t r3, int lane)
{
    uint32_t my = idx + (uint32_t)(lane & 15);
    int src = (int)((my >> 2) - base) & 31;
    uint32_t v0 = __shfl_sync(0xffffffffu, r0, src);
    uint32_t v1 = __shfl_sync(0xffffffffu, r1, src);
    uint32_t v2 = __shfl_sync(0xffffffffu, r2, src);
    uint32_t v3 = __shfl_sync(0xffffffffu, r3, src);
    uint32_t c = my & 3u;
    uint32_t v = c == 0 ? v0 : (c == 1 ? v1 : (c == 2 ? v2 : v3));
    float u = (lane & 15) < 12 ? bamf_u31_to_float(v >> 1) : 0.0f;
    u += __shfl_xor_sync(0xffffffffu, u, 1);
    u += __shfl_xor_sync(0xffffffffu, u, 2);
    u += __shfl_xor_sync(0xffffffffu, u, 4);
    u += __shfl_xor_sync(0xffffffffu, u, 8);
    return u - 6.0f;
}

/* Uniform in [0, 1) shared by the warps of a CTA in move-synchronous mode:
 * a 32-bit integer hash (the "lowbias32" xorshift-multiply finaliser,
 * applied twice) of (seed, group, step, which). */
__device__ __forceinline__ float shared_uniform(uint32_t seed, uint32_t grp, uint32_t step, uint32_t which)
{
    uint32_t x = seed * 0x9E3779B1u ^ grp * 0x85EBCA77u ^ (step * 2u + which) * 0xC2B2AE3Du;
    for (int r = 0; r < 2; ++r) {
        x ^= x >> 16;
        x *= 0x7feb352du;
        x ^= x >> 15;
        x *= 0x846ca68bu;
        x ^= x >> 16;
    }
    return (float)(x >> 8) * 5.9604644775390625e-08f;
}

/* (1 / A) / q(x, y) for the LEARNED birth proposal q = (learned + uniform)/2
 * on a box of area A; the learned part is the ROI's pixel running sum cdf
 * times the pixel's 16 sub-cell probabilities sub (16 cells per px^2). */
/* The learned position density at (x, y) per px^2 (pixel probability from
 * the running sum, sub-cell probability, 16 sub-cells per px^2); 0 outside
 * the ROI.  Call with the whole warp on the same arguments: lanes 0..15 load
 * the pixel's sub-cell probabilities and a butterfly sums them. */
static __device__ __noinline__ float learned_density(float x, float y, int X, int Y, int npix,
                                                     const float *__restrict__ cdf,
                                                     const float *__restrict__ sub)
{
    if (!(x >= 0.0f && y >= 0.0f && x < (float)X && y < (float)Y)) return 0.0f;
    const int lane = threadIdx.x & 31;
    int px = min((int)x, X - 1), py = min((int)y, Y - 1);
    int pix = py + px * Y;
    int sc = min((int)((y - (float)py) * 4.0f), 3) + 4 * min((int)((x - (float)px) * 4.0f), 3);
    float pp = __ldg(&cdf[pix]) - (pix > 0 ? __ldg(&cdf[pix - 1]) : 0.0f);
    const float *sp = sub + 16 * pix;
    const float v = lane < 16 ? __ldg(&sp[lane]) : 0.0f;
    float ps = v;
    for (int o = 1; o < 32; o <<= 1) ps += __shfl_xor_sync(0xffffffffu, ps, o);
    const float vs = __shfl_sync(0xffffffffu, v, sc);
    return (pp / __ldg(&cdf[npix - 1])) * (vs / ps) * 16.0f;
}

/* (1 / A) / q(x, y) for the birth mixture q = 1/2 learned + 1/2 uniform on
 * the extended box of area A. */
static __device__ __noinline__ float learned_q_ratio(float x, float y, int X, int Y, int npix, float A,
                                                     const float *__restrict__ cdf,
                                                     const float *__restrict__ sub)
{
    const float qa = learned_density(x, y, X, Y, npix, cdf, sub) * A; /* learned density times box area */
    return 1.0f / (0.5f * qa + 0.5f);
}

/* normpdf (LibRJMCMCreturn.hpp:19-21) with (float)sqrt(2.0f*pi), pi = 3.141592. */
template <bool EXACT>
static __device__ __noinline__ float normpdf_f(float x, float u, float s)
{
    const float sq2pi = (float)sqrt(2.0 * 3.141592);
    float d = x - u;
    return 1.0f / (sq2pi * s) * SMath<EXACT>::exp_(-d * d / (2.0f * s * s));
}

template <bool EXACT, bool NUM>
struct ChainWarp {
    typedef SMath<EXACT> MT;
    const SamplerConsts *K;
    const SamplerBatch *B;
    int lane;
    int roi;
    /* geometry */
    int X, Y, npix;
    int px_dx, px_dy; /* pixel p -> p+32 moves x by px_dx and y by px_dy (then wraps) */
    float sigma, Cst, MeanN;
    /* shared memory */
    float *D, *M, *Mt, *E, *NX, *NY;
    float *NXt, *NYt; /* exact mode: stencil rows of T (NX, NY hold A's) */
    int tsrc;         /* exact mode: the A slot T's emitter in this lane came from, -1 if changed */
    float *SXo, *SYo, *SXn, *SYn; /* fast mode: compact stencil rows */
    const float *scm; /* sCMOS: shared memory (exact) or global/null (fast) */
    /* sampled PSF (OptModel 1): [P0 y][P1 x][P2 y-sub][P3 x-sub], y fastest;
     * null for the Gaussian model */
    const float *psf;
    int pn0, pn01, pn012, ptot, pos;
    int *cnt, *cl;
    int rec_n[2];
    /* current state A (lane j = slot j) */
    int an;
    float aI, aX, aY;
    int aS;
    float aBG, aABG, aBBG;
    /* proposed state T */
    int tn;
    float tI, tX, tY;
    int tS;
    float tBG, tABG, tBBG;
    bool t_overflow;
    /* uniform stream */
    uint32_t seed, chain, idx, base;
    uint32_t r0, r1, r2, r3;
    /* phase */
    int is_burnin;
    float P[8];
    int entries;
    int overflow;
    int n_llr;
    /* incremental-model bookkeeping (fast mode) */
    uint32_t a_dirty, t_dirty;
    int llr_box; /* pixels the last likelihood pass changed: x0 | x1 << 8 | y0 << 16 | y1 << 24 */
    float pdf_aBG; /* fast mode: offset-prior density of aBG */
    /* move-synchronous mode: the jump sub-branch uniform comes from the CTA */
    bool use_shared_ub;
    float shared_ub;

    /* ---------------------------------------------------------- RNG */
    __device__ __forceinline__ void refill()
    {
        uint4 b = philox_block(base + (uint32_t)lane, seed, chain);
        r0 = b.x; r1 = b.y; r2 = b.z; r3 = b.w;
    }
    __device__ __forceinline__ float urand()
    {
        uint32_t blk = idx >> 2;
        if (blk - base >= 32u) {
            base = blk;
            refill();
        }
        uint32_t c = idx & 3u;
        uint32_t v = c == 0 ? r0 : (c == 1 ? r1 : (c == 2 ? r2 : r3));
        v = __shfl_sync(BAMF_FULL, v, (int)(blk - base));
        idx++;
        return bamf_u31_to_float(v >> 1);
    }
    /* Irwin-Hall sum of 12 uniforms (LibRJMCMCreturn.hpp:23-26).  Exact
     * mode adds them in draw order; fast mode has lanes 0..11 fetch the 12
     * draws at once and adds them in a butterfly (same distribution, other
     * rounding). */
    __device__ __forceinline__ float randn()
    {
        if (EXACT) {
            float t = 0;
            for (int k = 0; k < 12; ++k) t = t + urand();
            return t - 6.0f;
        }
        if (((idx + 11u) >> 2) - base >= 32u) {
            base = idx >> 2;
            refill();
        }
        float u = irwin_hall12(idx, base, r0, r1, r2, r3, lane);
        idx += 12u;
        return u;
    }

    /* ------------------------------------------------------ lane access */
    __device__ __forceinline__ float A_I(int k) const { return __shfl_sync(BAMF_FULL, aI, k); }
    __device__ __forceinline__ float A_X(int k) const { return __shfl_sync(BAMF_FULL, aX, k); }
    __device__ __forceinline__ float A_Y(int k) const { return __shfl_sync(BAMF_FULL, aY, k); }
    __device__ __forceinline__ int A_S(int k) const { return __shfl_sync(BAMF_FULL, aS, k); }
    __device__ __forceinline__ float T_I(int k) const { return __shfl_sync(BAMF_FULL, tI, k); }
    __device__ __forceinline__ int T_S(int k) const { return __shfl_sync(BAMF_FULL, tS, k); }

    __device__ __forceinline__ void setT(int k, float I, float x, float y)
    {
        if (lane == k) {
            tI = I;
            tX = x;
            tY = y;
            if (EXACT) tsrc = -1;
        }
        if (!EXACT) t_dirty |= 1u << k;
    }
    __device__ __forceinline__ void addT(float I, float x, float y, int s)
    {
        if (tn >= BAMF_NMAX) {
            t_overflow = true;
            return;
        }
        if (lane == tn) {
            tI = I;
            tX = x;
            tY = y;
            tS = s;
            if (EXACT) tsrc = -1;
        }
        if (!EXACT) t_dirty |= 1u << tn;
        tn++;
    }
    /* Emitters::remove (LibRJMCMC.cpp:478-490) */
    __device__ __forceinline__ void removeT(int id)
    {
        float vI = __shfl_down_sync(BAMF_FULL, tI, 1);
        float vX = __shfl_down_sync(BAMF_FULL, tX, 1);
        float vY = __shfl_down_sync(BAMF_FULL, tY, 1);
        int vS = __shfl_down_sync(BAMF_FULL, tS, 1);
        int vsrc = EXACT ? __shfl_down_sync(BAMF_FULL, tsrc, 1) : 0;
        if (lane >= id) {
            tI = vI; tX = vX; tY = vY; tS = vS;
            if (EXACT) tsrc = vsrc;
        }
        if (!EXACT) {
            uint32_t lo = t_dirty & ((1u << id) - 1u);
            uint32_t hi = id < 31 ? (t_dirty >> (id + 1)) << id : 0u;
            t_dirty = lo | hi;
        }
        tn--;
    }
    __device__ __forceinline__ void copyA2T()
    {
        tn = an; tI = aI; tX = aX; tY = aY; tS = aS;
        tBG = aBG; tABG = aABG; tBBG = aBBG;
        t_overflow = false;
        if (EXACT) tsrc = lane;
        if (!EXACT) {
            a_dirty = 0u;
            t_dirty = 0u;
        }
    }
    __device__ __forceinline__ void cinc(int k)
    {
        if (lane == 0) cnt[k]++;
    }

    /* Emitters::test (:492-514) with Bnd_out cast to int. */
    __device__ __forceinline__ bool testT() const
    {
        int bnd = (int)K->p.Bnd_out;
        bool bad = false;
        if (lane < tn)
            bad = (tI < 0.0f) || (tX < (float)(-bnd)) || (tY < (float)(-bnd)) ||
                  (tX > (float)(X + bnd)) || (tY > (float)(Y + bnd));
        return !__any_sync(BAMF_FULL, bad);
    }

    __device__ __forceinline__ float nsignalA() const
    {
        return (float)__popc(__ballot_sync(BAMF_FULL, lane < an && aS == 1));
    }

    /* ---------------------------------------------------- prior tables */
    __device__ __forceinline__ float findPDF(const DevStat &s, float I) const
    {
        if (EXACT) return stat_pdf(s.x, s.pdf, s.L, I);
        return stat_pdf_fast(s.x, s.pdf, s.L, s.inv_dx, I);
    }
    __device__ __forceinline__ float genRand(const DevStat &s)
    {
        float R = urand();
        if (EXACT) return stat_rand(s.ux, s.uc, s.nu, R);
        return stat_rand_warp(s.ux, s.uc, s.nu, R, lane);
    }
    __device__ __forceinline__ float sob(int signal, float I) const
    {
        const DevStat &s = signal == 1 ? K->sig : K->back;
        return findPDF(s, I);
    }
    __device__ __forceinline__ float normpdf(float x, float u, float s) const
    {
        return normpdf_f<EXACT>(x, u, s);
    }

    /* ------------------------------------------------ neighbour search */
    __device__ __forceinline__ uint32_t near_mask(int jj, float dmin) const
    {
        float xj = A_X(jj), yj = A_Y(jj);
        bool in = false;
        if (lane < an && lane != jj) {
            float dx = aX - xj, dy = aY - yj;
            float d;
            if (EXACT)
                d = (float)sqrt(dadd(dmul((double)dx, (double)dx), dmul((double)dy, (double)dy)));
            else
                d = sqrtf(dx * dx + dy * dy);
            in = d < dmin;
        }
        return __ballot_sync(BAMF_FULL, in);
    }
    static __device__ __forceinline__ int nth_bit(uint32_t m, int q)
    {
        for (int t = 0; t < q; ++t) m &= m - 1u;
        return __ffs(m) - 1;
    }
    /* Emitters::closest (:525-558). */
    __device__ __forceinline__ int closest(int jj, float dmin)
    {
        uint32_t m = near_mask(jj, dmin);
        int num = __popc(m);
        if (num > 0) {
            float Ua = urand();
            int mm = min((int)(Ua * (float)num), num - 1);
            return nth_bit(m, mm);
        }
        uint32_t others = (an >= 32 ? BAMF_FULL : ((1u << an) - 1u)) & ~(1u << jj);
        float Ua = urand();
        int mm = min((int)(Ua * (float)(an - 1)), an - 2);
        return nth_bit(others, mm);
    }
    /* Emitters::closestMulti (:615-650); picks go to cl[] in pick order. */
    __device__ __forceinline__ int closestMulti(int jj, float dmin)
    {
        uint32_t m = near_mask(jj, dmin);
        int num = __popc(m);
        int np = 0;
        if (num > 0) {
            float Ua = urand();
            int Np;
            if (Ua < 1.0f / (float)num) Np = num;
            else Np = min((int)(Ua * (float)num), num - 1);
            for (int n = 0; n < Np; ++n) {
                Ua = urand();
                int q = min((int)(Ua * (float)(num - n)), num - n - 1);
                int b = nth_bit(m, q);
                m &= ~(1u << b);
                if (lane == 0) cl[np] = b;
                np++;
            }
        }
        __syncwarp();
        return np;
    }

    /* ------------------------------------------------------------ model */
    /* Stencil + Model (:15-59) of a lane-distributed state, into out[]. */
    __device__ __forceinline__ void model_full(int n, float I, float Xv, float Yv, float BG, float ABG, float BBG,
                               float *out, float *nx, float *ny)
    {
        int totx = n * X, toty = n * Y;
#pragma unroll 1
        for (int b0 = 0; b0 < totx; b0 += 32) {
            int item = b0 + lane;
            int k = min(item / X, n - 1);
            int x = item - k * X;
            float Ik = __shfl_sync(BAMF_FULL, I, k);
            float Xk = __shfl_sync(BAMF_FULL, Xv, k);
            if (item < totx)
                nx[k * X + x] = Ik * 0.5f * (MT::erf_(((float)x - Xk + 1.0f) * Cst) -
                                             MT::erf_(((float)x - Xk) * Cst));
        }
#pragma unroll 1
        for (int b0 = 0; b0 < toty; b0 += 32) {
            int item = b0 + lane;
            int k = min(item / Y, n - 1);
            int y = item - k * Y;
            float Yk = __shfl_sync(BAMF_FULL, Yv, k);
            if (item < toty)
                ny[k * Y + y] = 0.5f * (MT::erf_(((float)y - Yk + 1.0f) * Cst) -
                                        MT::erf_(((float)y - Yk) * Cst));
        }
        __syncwarp();
        int x = lane / Y, y = lane - (lane / Y) * Y;
#pragma unroll 1
        for (int p = lane; p < npix; p += 32) {
            float m = BG + ABG * (float)x + BBG * (float)y + (scm ? scm[p] : 0.0f);
            for (int k = 0; k < n; ++k) m += nx[k * X + x] * ny[k * Y + y];
            out[p] = m;
            x += px_dx;
            y += px_dy;
            if (y >= Y) {
                y -= Y;
                x++;
            }
        }
        __syncwarp();
    }

    /* Exact mode, the proposal's model: as model_full for T, but the
     * stencil rows of the emitters the proposal left unchanged are copied
     * from A's rows (the same function of the same inputs, so the same
     * bits) instead of evaluated again; only changed or new emitters pay
     * the erf evaluations.  Rows go to NXt / NYt. */
    __device__ __forceinline__ void model_cached(int n, float I, float Xv, float Yv, float BG, float ABG, float BBG,
                                                 float *out)
    {
        int totx = n * X, toty = n * Y;
#pragma unroll 1
        for (int b0 = 0; b0 < totx; b0 += 32) {
            int item = b0 + lane;
            int k = min(item / X, n - 1);
            int x = item - k * X;
            float Ik = __shfl_sync(BAMF_FULL, I, k);
            float Xk = __shfl_sync(BAMF_FULL, Xv, k);
            int src = __shfl_sync(BAMF_FULL, tsrc, k);
            if (item < totx)
                NXt[k * X + x] = src >= 0 ? NX[src * X + x]
                                          : Ik * 0.5f * (MT::erf_(((float)x - Xk + 1.0f) * Cst) -
                                                         MT::erf_(((float)x - Xk) * Cst));
        }
#pragma unroll 1
        for (int b0 = 0; b0 < toty; b0 += 32) {
            int item = b0 + lane;
            int k = min(item / Y, n - 1);
            int y = item - k * Y;
            float Yk = __shfl_sync(BAMF_FULL, Yv, k);
            int src = __shfl_sync(BAMF_FULL, tsrc, k);
            if (item < toty)
                NYt[k * Y + y] = src >= 0 ? NY[src * Y + y]
                                          : 0.5f * (MT::erf_(((float)y - Yk + 1.0f) * Cst) -
                                                    MT::erf_(((float)y - Yk) * Cst));
        }
        __syncwarp();
        int x = lane / Y, y = lane - (lane / Y) * Y;
#pragma unroll 1
        for (int p = lane; p < npix; p += 32) {
            float m = BG + ABG * (float)x + BBG * (float)y + (scm ? scm[p] : 0.0f);
            for (int k = 0; k < n; ++k) m += NXt[k * X + x] * NYt[k * Y + y];
            out[p] = m;
            x += px_dx;
            y += px_dy;
            if (y >= Y) {
                y -= Y;
                x++;
            }
        }
        __syncwarp();
    }

    /* Fast mode: stencil rows of the emitters a proposal changes, compact:
     * row q of SXo/SYo is the old stencil of the q-th slot of a_dirty (from
     * A), row q of SXn/SYn the new stencil of the q-th slot of t_dirty (from
     * T). */
    __device__ __forceinline__ void stencil_rows(int na, int nt)
    {
        const int XY = X + Y, nr = na + nt;
        /* G rows per 32-lane pass when a row (X + Y entries) fits in 32
         * lanes, else one row at a time over ceil(XY / 32) passes */
        const int G = XY <= 32 ? 32 / XY : 1;
        const int rg = XY <= 32 ? lane / XY : 0;
        const int c0 = XY <= 32 ? lane - rg * XY : lane;
#pragma unroll 1
        for (int r0 = 0; r0 < nr; r0 += G) {
            int r = min(r0 + rg, nr - 1);
            bool isnew = r >= na;
            int q = isnew ? r - na : r;
            int k = nth_bit(isnew ? t_dirty : a_dirty, q);
            /* a shuffle returns the source lane's value, so fetch both
             * states and select here (lanes of one pass may read rows of
             * different states) */
            float Ia = __shfl_sync(BAMF_FULL, aI, k), It = __shfl_sync(BAMF_FULL, tI, k);
            float Xa = __shfl_sync(BAMF_FULL, aX, k), Xt = __shfl_sync(BAMF_FULL, tX, k);
            float Ya = __shfl_sync(BAMF_FULL, aY, k), Yt = __shfl_sync(BAMF_FULL, tY, k);
            float Ik = isnew ? It : Ia, Xk = isnew ? Xt : Xa, Yk = isnew ? Yt : Ya;
            bool on = rg < G && r0 + rg < nr;
            float *sxr = (isnew ? SXn : SXo) + q * X, *syr = (isnew ? SYn : SYo) + q * Y;
#pragma unroll 1
            for (int c = c0; c < XY; c += 32) {
                bool isx = c < X;
                int cc = isx ? c : c - X;
                float mu = isx ? Xk : Yk;
                float v = 0.5f * (MT::erf_(((float)cc - mu + 1.0f) * Cst) - MT::erf_(((float)cc - mu) * Cst));
                if (on) {
                    if (isx) sxr[cc] = Ik * v;
                    else syr[cc] = v;
                }
                if (XY <= 32) break;
            }
        }
        __syncwarp();
    }

    /* Fast mode: out = background plane + sCMOS + sum of the state's emitter
     * stencils, one emitter at a time (its rows go through SXn/SYn row 0). */
    __device__ __forceinline__ void model_stream(int n, float I, float Xv, float Yv, float BG, float ABG,
                                                 float BBG, float *out)
    {
        int x = lane / Y, y = lane - (lane / Y) * Y;
#pragma unroll 1
        for (int p = lane; p < npix; p += 32) {
            out[p] = BG + ABG * (float)x + BBG * (float)y + (scm ? scm[p] : 0.0f);
            x += px_dx;
            y += px_dy;
            if (y >= Y) {
                y -= Y;
                x++;
            }
        }
#pragma unroll 1
        for (int k = 0; k < n; ++k) {
            float Ik = __shfl_sync(BAMF_FULL, I, k), Xk = __shfl_sync(BAMF_FULL, Xv, k);
            float Yk = __shfl_sync(BAMF_FULL, Yv, k);
            __syncwarp();
#pragma unroll 1
            for (int c = lane; c < X + Y; c += 32) {
                bool isx = c < X;
                int cc = isx ? c : c - X;
                float mu = isx ? Xk : Yk;
                float v = 0.5f * (MT::erf_(((float)cc - mu + 1.0f) * Cst) - MT::erf_(((float)cc - mu) * Cst));
                if (isx) SXn[cc] = Ik * v;
                else SYn[cc] = v;
            }
            __syncwarp();
            x = lane / Y;
            y = lane - (lane / Y) * Y;
#pragma unroll 1
            for (int p = lane; p < npix; p += 32) {
                out[p] += SXn[x] * SYn[y];
                x += px_dx;
                y += px_dy;
                if (y >= Y) {
                    y -= Y;
                    x++;
                }
            }
        }
        __syncwarp();
    }

    /* ------------------------------------------ sampled-PSF model */
    /* NumModel (:67-170) places emitter (x, y) on four planes of the sampled
     * PSF: pixel (xx, yy) of the ROI reads flat index b_i + yy + xx P0 of
     * plane i and blends them bilinearly with weights wx (x) and wy (y).
     * Exact mode repeats the reference's double arithmetic; fast mode takes
     * the same steps in float. */
    struct NumPlace {
        int b1, b2, b3, b4;
        float wx, wy;
    };
    __device__ __forceinline__ NumPlace num_place(float xf, float yf) const
    {
        const int c0 = pn0 / 2;
        int sx, sy, ix, iy;
        NumPlace q;
        if (EXACT) {
            const double xd = (double)xf, yd = (double)yf, os = (double)pos;
            const double fx = dadd(xd, -floor(xd)), fy = dadd(yd, -floor(yd));
            sx = (int)ceil(dadd((double)c0, -xd));
            ix = (int)floor(dmul(os, fx));
            sy = (int)ceil(dadd((double)c0, -yd));
            iy = (int)floor(dmul(os, fy));
            q.wy = (float)dadd(1.0, -dmul(dadd(fy, -__ddiv_rn((double)iy, os)), os));
            q.wx = (float)dadd(1.0, -dmul(dadd(fx, -__ddiv_rn((double)ix, os)), os));
        } else {
            const float os = (float)pos;
            const float fx = xf - floorf(xf), fy = yf - floorf(yf);
            sx = (int)ceilf((float)c0 - xf);
            ix = (int)floorf(os * fx);
            sy = (int)ceilf((float)c0 - yf);
            iy = (int)floorf(os * fy);
            q.wy = 1.0f - (fy * os - (float)iy);
            q.wx = 1.0f - (fx * os - (float)ix);
        }
        int sx2 = sx, ix2 = ix + 1, sy2 = sy, iy2 = iy + 1;
        if (ix == pos - 1) {
            sx2 = sx - 1;
            ix2 = 0;
        }
        if (iy == pos - 1) {
            sy2 = sy - 1;
            iy2 = 0;
        }
        q.b1 = sy + sx * pn0 + iy * pn01 + ix * pn012;
        q.b2 = sy + sx2 * pn0 + iy * pn01 + ix2 * pn012;
        q.b3 = sy2 + sx * pn0 + iy2 * pn01 + ix * pn012;
        q.b4 = sy2 + sx2 * pn0 + iy2 * pn01 + ix2 * pn012;
        return q;
    }
    /* a flat index outside the array reads its last element (:131-157) */
    __device__ __forceinline__ float psf_at(int i) const
    {
        return psf[(i >= ptot || i < 0) ? ptot - 1 : i];
    }
    /* the blended PSF value of pixel offset o = yy + xx P0 */
    __device__ __forceinline__ float num_value(const NumPlace &q, int o) const
    {
        float a = q.wx * psf_at(q.b1 + o) + (1.0f - q.wx) * psf_at(q.b2 + o);
        float b = q.wx * psf_at(q.b3 + o) + (1.0f - q.wx) * psf_at(q.b4 + o);
        return q.wy * a + (1.0f - q.wy) * b;
    }
    __device__ __forceinline__ static NumPlace shfl_place(const NumPlace &q, int k)
    {
        NumPlace r;
        r.b1 = __shfl_sync(BAMF_FULL, q.b1, k);
        r.b2 = __shfl_sync(BAMF_FULL, q.b2, k);
        r.b3 = __shfl_sync(BAMF_FULL, q.b3, k);
        r.b4 = __shfl_sync(BAMF_FULL, q.b4, k);
        r.wx = __shfl_sync(BAMF_FULL, q.wx, k);
        r.wy = __shfl_sync(BAMF_FULL, q.wy, k);
        return r;
    }

    /* NumModel of a lane-distributed state into out[] (both modes: the
     * background plane, then the emitters in slot order, per pixel). */
    __device__ __forceinline__ void model_num(int n, float I, float Xv, float Yv, float BG, float ABG, float BBG,
                                              float *out)
    {
        NumPlace q = num_place(lane < n ? Xv : 0.0f, lane < n ? Yv : 0.0f);
#pragma unroll 1
        for (int b0 = 0; b0 < npix; b0 += 32) {
            const int p = b0 + lane;
            const bool v = p < npix;
            const int x = p / Y, y = p - x * Y;
            float m = v ? BG + ABG * (float)x + BBG * (float)y + (scm ? scm[p] : 0.0f) : 0.0f;
            const int o = y + x * pn0;
#pragma unroll 1
            for (int k = 0; k < n; ++k) {
                NumPlace r = shfl_place(q, k);
                float Ik = __shfl_sync(BAMF_FULL, I, k);
                if (v) m = m + Ik * num_value(r, o);
            }
            if (v) out[p] = m;
        }
        __syncwarp();
    }

    /* Fast mode, sampled PSF: Mt = M + the background change - the changed
     * emitters of A + the changed emitters of T (lane q < na + nt holds
     * changed slot q, intensity negated for A's); returns the pixel sum of
     * D (ln Mt - ln M) - (Mt - M). */
    __device__ __forceinline__ float llr_num_fast(int na, int nt)
    {
        const float LN2 = 0.69314718f;
        const int nr = na + nt;
        const bool isnew = lane >= na;
        const int qq = isnew ? lane - na : lane;
        int k = lane < nr ? nth_bit(isnew ? t_dirty : a_dirty, qq) : 0;
        float Ia = __shfl_sync(BAMF_FULL, aI, k), It = __shfl_sync(BAMF_FULL, tI, k);
        float Xa = __shfl_sync(BAMF_FULL, aX, k), Xt = __shfl_sync(BAMF_FULL, tX, k);
        float Ya = __shfl_sync(BAMF_FULL, aY, k), Yt = __shfl_sync(BAMF_FULL, tY, k);
        const float Iq = lane < nr ? (isnew ? It : -Ia) : 0.0f;
        NumPlace q = num_place(isnew ? Xt : Xa, isnew ? Yt : Ya);
        const float dBG = tBG - aBG, dABG = tABG - aABG, dBBG = tBBG - aBBG;
        float acc = 0.0f;
#pragma unroll 1
        for (int b0 = 0; b0 < npix; b0 += 32) {
            const int p = b0 + lane;
            const bool v = p < npix;
            const int x = p / Y, y = p - x * Y;
            float d = dBG + dABG * (float)x + dBBG * (float)y;
            const int o = y + x * pn0;
#pragma unroll 1
            for (int r = 0; r < nr; ++r) {
                NumPlace g = shfl_place(q, r);
                float Ir = __shfl_sync(BAMF_FULL, Iq, r);
                if (v) d += Ir * num_value(g, o);
            }
            if (v) {
                float mt = M[p] + d;
                Mt[p] = mt;
                acc += D[p] * (__log2f(mt) - __log2f(M[p])) * LN2 - d;
            }
        }
        return acc;
    }

    /* likelihood_ratio (:1650-1686).  M always holds Model(A). */
    __device__ __forceinline__ float llr()
    {
        n_llr++;
        if (EXACT) {
            if constexpr (NUM) model_num(tn, tI, tX, tY, tBG, tABG, tBBG, Mt);
            else model_cached(tn, tI, tX, tY, tBG, tABG, tBBG, Mt);
            for (int p = lane; p < npix; p += 32)
                E[p] = M[p] - Mt[p] + D[p] * MT::log_(Mt[p] / M[p]);
            __syncwarp();
            float tmp = 0.0f;
            if (lane == 0)
                for (int p = 0; p < npix; ++p) tmp += E[p];
            tmp = __shfl_sync(BAMF_FULL, tmp, 0);
            return MT::exp_(tmp);
        } else {
            /* Mt = M + background delta - old stencils of A's changed slots
             *        + new stencils of T's changed slots;
             * sum over pixels of (M - Mt) + D (ln Mt - ln M) */
            const float LN2 = 0.69314718f;
            int na = __popc(a_dirty), nt = __popc(t_dirty);
            float acc = 0.0f;
            if constexpr (NUM) {
                llr_box = full_box();
                if (na <= FAST_ROWS && nt <= FAST_ROWS) {
                    acc = llr_num_fast(na, nt);
                } else {
                    model_num(tn, tI, tX, tY, tBG, tABG, tBBG, Mt);
#pragma unroll 1
                    for (int p = lane; p < npix; p += 32) {
                        float mt = Mt[p];
                        acc += D[p] * (__log2f(mt) - __log2f(M[p])) * LN2 - (mt - M[p]);
                    }
                }
            } else {
                if (na <= FAST_ROWS && nt <= FAST_ROWS) {
                    stencil_rows(na, nt);
                    const int nr = na + nt;
                    /* Support box: unless the background changes, a pixel
                     * outside the union of the changed rows' nonzero x- and
                     * y-stencil entries has d = 0 exactly (Mt = M, a zero
                     * term), so the pass covers only the box.  Stencils of
                     * sigma ~1.3 vanish in float ~7 px from the emitter. */
                    int x0 = 0, x1 = X - 1, y0 = 0, y1 = Y - 1;
                    if (tBG == aBG && tABG == aABG && tBBG == aBBG) {
                        bool nzx = false, nzy = false;
#pragma unroll 1
                        for (int q = 0; q < nr; ++q) {
                            const bool old = q < na;
                            const int qq = old ? q : q - na;
                            nzx |= lane < X && (old ? SXo : SXn)[qq * X + lane] != 0.0f;
                            nzy |= lane < Y && (old ? SYo : SYn)[qq * Y + lane] != 0.0f;
                        }
                        const uint32_t mx = __ballot_sync(BAMF_FULL, nzx), my = __ballot_sync(BAMF_FULL, nzy);
                        if (mx == 0u || my == 0u) {
                            llr_box = 1; /* empty: Mt = M everywhere, LLR = 1 */
                            return 1.0f;
                        }
                        x0 = __ffs(mx) - 1;
                        x1 = 31 - __clz(mx);
                        y0 = __ffs(my) - 1;
                        y1 = 31 - __clz(my);
                    }
                    llr_box = x0 | (x1 << 8) | (y0 << 16) | (y1 << 24);
                    /* lane -> row y = y0 + lane mod h of column x0 + lane / h
                     * (h the box height); a pass covers 32 / h columns.  The
                     * model change of a pixel is bg delta + sum_q w_q(y)
                     * SX_q[x] over the changed rows q (old rows with weight
                     * -SYo, new with +SYn); each lane holds its first four
                     * weights in registers. */
                    const int h = y1 - y0 + 1;
                    const int yl = y0 + lane % h, xo = lane / h, R = 32 / h;
                    float w[4];
                    const float *sx[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        bool old = q < na;
                        int qq = old ? q : q - na;
                        w[q] = q < nr ? (old ? -SYo[qq * Y + yl] : SYn[qq * Y + yl]) : 0.0f;
                        sx[q] = old ? SXo + qq * X : SXn + qq * X;
                    }
                    const float base = (tBG - aBG) + (tBBG - aBBG) * (float)yl, dABG = tABG - aABG;
                    if (xo < R) {
#pragma unroll 1
                        for (int xx = x0 + xo; xx <= x1; xx += R) {
                            float d = base + dABG * (float)xx;
                            if (nr > 0) d += w[0] * sx[0][xx];
                            if (nr > 1) d += w[1] * sx[1][xx];
                            if (nr > 2) d += w[2] * sx[2][xx];
                            if (nr > 3) d += w[3] * sx[3][xx];
                            for (int q = 4; q < nr; ++q)
                                d += q < na ? -SXo[q * X + xx] * SYo[q * Y + yl]
                                            : SXn[(q - na) * X + xx] * SYn[(q - na) * Y + yl];
                            int p = yl + Y * xx;
                            float mt = M[p] + d;
                            Mt[p] = mt;
                            acc += D[p] * (__log2f(mt) - __log2f(M[p])) * LN2 - d;
                        }
                    }
                } else {
                    model_stream(tn, tI, tX, tY, tBG, tABG, tBBG, Mt);
                    llr_box = full_box();
#pragma unroll 1
                    for (int p = lane; p < npix; p += 32) {
                        float mt = Mt[p];
                        acc += D[p] * (__log2f(mt) - __log2f(M[p])) * LN2 - (mt - M[p]);
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(BAMF_FULL, acc, o);
            return MT::exp_(acc);
        }
    }

    /* fast mode: fold the accepted proposal into M (Mt differs from M only
     * inside the box of the last likelihood pass) */
    __device__ __forceinline__ int full_box() const { return (X - 1) << 8 | (Y - 1) << 24; }
    __device__ __forceinline__ void commit_fast()
    {
        const int x0 = llr_box & 255, x1 = (llr_box >> 8) & 255, y0 = (llr_box >> 16) & 255, y1 = llr_box >> 24;
        if (x0 <= x1) {
            const int h = y1 - y0 + 1, R = 32 / h, yy = y0 + lane % h, xo = lane / h;
            if (xo < R) {
#pragma unroll 1
                for (int xx = x0 + xo; xx <= x1; xx += R) M[yy + Y * xx] = Mt[yy + Y * xx];
            }
        }
        __syncwarp();
    }

    __device__ __forceinline__ void accept_T()
    {
        if (!EXACT) {
            commit_fast();
            if (tBG != aBG) pdf_aBG = findPDF(K->off, tBG);
        }
        an = tn; aI = tI; aX = tX; aY = tY; aS = tS;
        aBG = tBG; aABG = tABG; aBBG = tBBG;
        if (EXACT) {
            float *t = M;
            M = Mt;
            Mt = t;
            t = NX; NX = NXt; NXt = t;
            t = NY; NY = NYt; NYt = t;
        }
    }

    /* Full rebuild of M. */
    __device__ __forceinline__ void rebuild_model()
    {
        if (EXACT) {
            if constexpr (NUM) model_num(an, aI, aX, aY, aBG, aABG, aBBG, M);
            else model_full(an, aI, aX, aY, aBG, aABG, aBBG, M, NX, NY);
        } else {
            /* with a drift output, a periodic rebuild goes to Mt (free
             * between proposals) first, to measure how far the incrementally
             * updated M has moved from the model of its state */
            const bool chk = B->model_drift != nullptr && entries > 0;
            float *dst = chk ? Mt : M;
            if constexpr (NUM) model_num(an, aI, aX, aY, aBG, aABG, aBBG, dst);
            else model_stream(an, aI, aX, aY, aBG, aABG, aBBG, dst);
            __syncwarp();
            if (chk) {
                float d = 0.0f;
                for (int p = lane; p < npix; p += 32) {
                    const float m = Mt[p];
                    d = fmaxf(d, fabsf(M[p] - m) / m);
                    M[p] = m;
                }
                for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(BAMF_FULL, d, o));
                /* non-negative floats order like their bit patterns */
                if (lane == 0) atomicMax((int *)&B->model_drift[roi], __float_as_int(d));
                __syncwarp();
            }
        }
    }

    /* ------------------------------------------------------- recording */
    __device__ __forceinline__ void record_one(int w, int n, float I, float x, float y, int s, float BG, float ABG,
                               float BBG, float LLR, float PR, int type, int acc)
    {
        bamf_chain *ch = &B->chains[2 * roi + w];
        int e = entries;
        if (e >= ch->capacity_entries) return;
        if (lane == 0) {
            ch->N[e] = n; ch->LLR[e] = LLR; ch->PR[e] = PR; ch->JumpType[e] = type;
            ch->Accepted[e] = acc; ch->BG[e] = BG; ch->ABG[e] = ABG; ch->BBG[e] = BBG;
        }
        int rc = rec_n[w];
        int nrec = n < 1 ? 1 : n;
        if (rc + nrec <= ch->capacity_records) {
            if (n < 1) {
                if (lane == 0) {
                    ch->Index[rc] = e + 1; ch->Photons[rc] = 0.0f; ch->X[rc] = -100.0f;
                    ch->Y[rc] = -100.0f; ch->Signal[rc] = -1;
                }
            } else if (lane < n) {
                ch->Index[rc + lane] = e + 1;
                ch->Photons[rc + lane] = I;
                ch->X[rc + lane] = x + K->p.DriftX;
                ch->Y[rc + lane] = y + K->p.DriftY;
                ch->Signal[rc + lane] = s;
            }
        }
        rec_n[w] = rc + nrec;
    }

    /* mean X of the Signal==1 emitters of A (NaN when none) into x_trace */
    __device__ __forceinline__ void record_x()
    {
        bool on = lane < an && aS == 1;
        float sx = on ? aX : 0.0f;
        for (int o = 16; o > 0; o >>= 1) sx += __shfl_xor_sync(BAMF_FULL, sx, o);
        int ns = __popc(__ballot_sync(BAMF_FULL, on));
        if (lane == 0)
            B->x_trace[(int64_t)roi * B->x_cap + entries] = ns > 0 ? sx / (float)ns : __int_as_float(0x7fc00000);
    }

    /* thinned state record: entry, Signal==1 count, BG, ABG, BBG, then X, Y,
     * I of the Signal==1 emitters in slot order (NaN past the count) */
    __device__ __forceinline__ void record_pos()
    {
        float *rec = B->pos_trace + ((int64_t)roi * B->pos_len + entries / B->pos_thin) * BAMF_POS_RECORD;
        bool on = lane < an && aS == 1;
        uint32_t m = __ballot_sync(BAMF_FULL, on);
        int rank = __popc(m & ((1u << lane) - 1u));
        int ns = __popc(m);
        if (lane == 0) {
            rec[0] = (float)entries;
            rec[1] = (float)ns;
            rec[2] = aBG;
            rec[3] = aABG;
            rec[4] = aBBG;
        }
        if (lane < BAMF_POS_SLOTS) {
            const float nan = __int_as_float(0x7fc00000);
            rec[5 + lane] = nan;
            rec[5 + BAMF_POS_SLOTS + lane] = nan;
            rec[5 + 2 * BAMF_POS_SLOTS + lane] = nan;
        }
        __syncwarp();
        if (on && rank < BAMF_POS_SLOTS) {
            rec[5 + rank] = aX;
            rec[5 + BAMF_POS_SLOTS + rank] = aY;
            rec[5 + 2 * BAMF_POS_SLOTS + rank] = aI;
        }
    }

    /* RJMCMCChain::addEmitters on Chain (A) and Chain_Test (T). */
    __device__ __forceinline__ void record2(float LLR, float PR, int type, int acc)
    {
        if (B->nsig_trace && entries < B->trace_cap) {
            int ns = __popc(__ballot_sync(BAMF_FULL, lane < an && aS == 1));
            if (lane == 0) B->nsig_trace[(int64_t)roi * B->trace_cap + entries] = (uint8_t)(an < 1 ? 0 : ns);
        }
        if (B->x_trace && entries < B->x_cap) record_x();
        if (B->pos_trace && entries % B->pos_thin == 0 && entries / B->pos_thin < B->pos_len) record_pos();
        if (B->chains) {
            record_one(0, an, aI, aX, aY, aS, aBG, aABG, aBBG, LLR, PR, type, acc);
            record_one(1, tn, tI, tX, tY, tS, tBG, tABG, tBBG, LLR, PR, type, acc);
        }
        entries++;
    }

    /* RJMCMC::update_grids (:1629-1648). */
    __device__ __forceinline__ void update_grids()
    {
        if (is_burnin || !B->pgrid) return;
        int Z = K->p.Grid_Zoom;
        if (lane < an) {
            /* the float sum with 0.5 is exact for |coordinate| < 2^22: fast
             * mode rounds as the reference's double sum does */
            const float gx = (float)Z * (aX + K->p.DriftX), gy = (float)Z * (aY + K->p.DriftY);
            int x = EXACT ? (int)floor(dadd((double)gx, 0.5)) : (int)floorf(gx + 0.5f);
            int y = EXACT ? (int)floor(dadd((double)gy, 0.5)) : (int)floorf(gy + 0.5f);
            float *gb = aS == 1 ? B->pgrid : B->pback;
            if (gb && x >= 0 && x < X * Z && y >= 0 && y < Y * Z && aI > K->p.Icutoff) {
                /* grid slot (ROIs sharing one accumulate) and column stride */
                int64_t slot = B->grid_slot ? (int64_t)B->grid_slot[roi] : (int64_t)roi;
                int64_t ld = B->grid_ld > 0 ? (int64_t)B->grid_ld : (int64_t)Y * Z;
                atomicAdd(&gb[slot * B->grid_stride + (int64_t)x * ld + y], 1.0f);
            }
        }
    }


    /* ------------------------------------------------------------ moves */
    /* Every move is split in two: propose_*() consumes the move's uniforms,
     * builds T and returns what happens next; finish_*() turns the
     * likelihood ratio into the move's posterior ratio (no uniforms).  The
     * likelihood ratio, the accept draw, the commit and the chain record are
     * then one shared code path in step(), in the reference's order
     * (proposal draws, test, likelihood_ratio, priors, accept draw). */
    enum { ACT_SKIP = 0, ACT_GRIDS = 1, ACT_REJECT = 2, ACT_EVAL = 3 };
    enum { MV_JUMP, MV_SPLIT, MV_MERGE, MV_BIRTH, MV_DEATH, MV_GSPLIT, MV_GMERGE };
    /* pending proposal between propose and finish */
    int pk_move, pk_type, pk_c1, pk_c2, pk_i0, pk_i1, pk_i2;
    float pk_f0, pk_f1, pk_f2, pk_f3, pk_f4, pk_f5;

    /* RJMCMC::jump (:752-970) up to the likelihood ratio. */
    __device__ __forceinline__ int propose_jump()
    {
        cinc(C_N_jump);
        int type = 1;
        float PrI = 1.0f, IPDF, IPDFtest;
        copyA2T();
        if (an < 1) return ACT_SKIP;
        float Ua = urand();
        int nn = min((int)(Ua * (float)tn), tn - 1);
        float Ub = use_shared_ub ? shared_ub : urand();
        const bamf_mcmc_params &p = K->p;
        if (Ub < 0.25f) {
            type = 2;
            tBG = tBG + p.BG_std * randn();
            tABG = tABG + p.ABBG_std * randn();
            tBBG = tBBG + p.ABBG_std * randn();
        } else if (Ub < 0.50f && Ub >= 0.25f) {
            if (an < 2) return ACT_SKIP;
            type = 10;
            int Np = closestMulti(nn, 2 * sigma);
            if (Np == 0) return ACT_SKIP;
            float I0 = A_I(nn);
            for (int i = 0; i < Np; ++i) I0 = I0 + A_I(cl[i]);
            float II0 = 0, XI0 = 0, YI0 = 0, XII0 = 0, YII0 = 0;
            for (int i = 0; i < Np; ++i) {
                int c = cl[i];
                float aIc = A_I(c), aXc = A_X(c), aYc = A_Y(c);
                int aSc = A_S(c);
                float nX, nY, nI;
                if (aSc == 1) {
                    nX = aXc + p.X_stdFg * randn();
                    nY = aYc + p.X_stdFg * randn();
                    nI = (I0 / (float)(Np + 1)) * (0.15f * randn() + 1.0f);
                    IPDFtest = findPDF(K->sig, nI);
                    IPDF = findPDF(K->sig, aIc);
                } else {
                    nX = aXc + p.X_stdBg * randn();
                    nY = aYc + p.X_stdBg * randn();
                    nI = (I0 / (float)(Np + 1)) * (0.15f * randn() + 1.0f);
                    IPDFtest = findPDF(K->back, nI);
                    IPDF = findPDF(K->back, aIc);
                }
                PrI = PrI * IPDFtest / IPDF;
                setT(c, nI, nX, nY);
                if (!EXACT) a_dirty |= 1u << c;
                XI0 = XI0 + aIc * aXc;
                YI0 = YI0 + aIc * aYc;
                XII0 = XII0 + nI * nX;
                YII0 = YII0 + nI * nY;
                II0 = II0 + nI;
            }
            float aIn = A_I(nn), aXn = A_X(nn), aYn = A_Y(nn);
            int aSn = A_S(nn);
            float tIn = I0 - II0;
            float tXn = (XI0 + aIn * aXn - XII0) / tIn;
            float tYn = (YI0 + aIn * aYn - YII0) / tIn;
            setT(nn, tIn, tXn, tYn);
            if (!EXACT) a_dirty |= 1u << nn;
            IPDFtest = sob(aSn, tIn);
            IPDF = sob(aSn, aIn);
            PrI = PrI * IPDFtest / IPDF;
        } else if (Ub >= 0.5f && Ub < 0.75f) {
            type = 3;
            int NN = closestMulti(nn, 2 * sigma);
            if (lane == 0) cl[NN] = nn;
            __syncwarp();
            NN++;
            for (int i = 0; i < NN; ++i) {
                int c = cl[i];
                float aIc = A_I(c);
                int aSc = A_S(c);
                float cI = T_I(c);
                float cX = __shfl_sync(BAMF_FULL, tX, c), cY = __shfl_sync(BAMF_FULL, tY, c);
                float nI, nX, nY;
                if (aSc == 1) {
                    cinc(C_N_jumpFg);
                    nI = cI + p.I_stdFg * randn();
                    nX = cX + p.X_stdFg * randn();
                    nY = cY + p.X_stdFg * randn();
                    IPDFtest = findPDF(K->sig, nI);
                    IPDF = findPDF(K->sig, aIc);
                } else {
                    cinc(C_N_jumpBg);
                    nI = cI + p.I_stdBg * randn();
                    nX = cX + p.X_stdBg * randn();
                    nY = cY + p.X_stdBg * randn();
                    IPDFtest = findPDF(K->back, nI);
                    IPDF = findPDF(K->back, aIc);
                }
                PrI = PrI * IPDFtest / IPDF;
                setT(c, nI, nX, nY);
                if (!EXACT) a_dirty |= 1u << c;
            }
        } else {
            float aIn = A_I(nn), aXn = A_X(nn), aYn = A_Y(nn);
            int aSn = A_S(nn);
            float nI, nX, nY;
            if (!EXACT && K->proposal == BAMF_PROPOSAL_LEARNED && urand() < 0.25f) {
                /* LEARNED relocation (no reference counterpart): an
                 * independence proposal of the emitter's position from the
                 * birth mixture q = 1/2 learned + 1/2 uniform on the extended
                 * box, intensity kept; Hastings factor q(old) / q(new) =
                 * birth_q_ratio(new) / birth_q_ratio(old), position prior
                 * uniform on the box, so the target is unchanged for any q */
                cinc(aSn == 1 ? C_N_jumpFg : C_N_jumpBg);
                birth_position(&nX, &nY);
                setT(nn, aIn, nX, nY);
                if (!EXACT) a_dirty |= 1u << nn;
                pk_move = MV_JUMP;
                pk_type = type;
                pk_f0 = birth_q_ratio(nX, nY) / birth_q_ratio(aXn, aYn);
                pk_c1 = C_A_jump;
                pk_c2 = aSn == 1 ? C_A_jumpFg : C_A_jumpBg;
                return testT() ? ACT_EVAL : ACT_REJECT;
            }
            if (aSn == 1) {
                cinc(C_N_jumpFg);
                nI = aIn + p.I_stdFg * randn();
                nX = aXn + p.X_stdFg * randn();
                nY = aYn + p.X_stdFg * randn();
                IPDFtest = findPDF(K->sig, nI);
                IPDF = findPDF(K->sig, aIn);
            } else {
                cinc(C_N_jumpBg);
                nI = aIn + p.I_stdBg * randn();
                nX = aXn + p.X_stdBg * randn();
                nY = aYn + p.X_stdBg * randn();
                IPDFtest = findPDF(K->back, nI);
                IPDF = findPDF(K->back, aIn);
            }
            PrI = IPDFtest / IPDF;
            setT(nn, nI, nX, nY);
            if (!EXACT) a_dirty |= 1u << nn;
        }
        pk_move = MV_JUMP;
        pk_type = type;
        pk_f0 = PrI;
        pk_c1 = C_A_jump;
        pk_c2 = A_S(nn) == 1 ? C_A_jumpFg : C_A_jumpBg;
        return testT() ? ACT_EVAL : ACT_REJECT;
    }
    __device__ __forceinline__ float finish_jump(float LLR)
    {
        if (!EXACT) {
            /* fast: the offset prior of the current BG is cached, and the
             * factors of an unchanged BG / slope are 1 (x / x, exp(0)) */
            float BgPDFtest = tBG == aBG ? pdf_aBG : findPDF(K->off, tBG);
            float PrBg = BgPDFtest / pdf_aBG;
            if (tBBG != aBBG) PrBg *= MT::exp_(-(tBBG * tBBG - aBBG * aBBG) / 2.0f);
            if (tABG != aABG) PrBg *= MT::exp_(-(tABG * tABG - aABG * aABG) / 2.0f);
            return LLR * pk_f0 * PrBg;
        }
        float BgPDF = findPDF(K->off, aBG);
        float BgPDFtest = findPDF(K->off, tBG);
        float PrBg = (BgPDFtest / BgPDF) * MT::exp_(-(tBBG * tBBG - aBBG * aBBG) / 2.0f) *
                     MT::exp_(-(tABG * tABG - aABG * aABG) / 2.0f);
        return LLR * pk_f0 * PrBg;
    }

    /* RJMCMC::split (:972-1109). */
    __device__ __forceinline__ int propose_split()
    {
        cinc(C_N_split);
        copyA2T();
        if (an < 1) return ACT_SKIP;
        const bamf_mcmc_params &p = K->p;
        float Ua = urand();
        int jj = min((int)floorf((float)an * Ua), an - 1);
        float Ijp = A_I(jj), mux = A_X(jj), muy = A_Y(jj);
        int BF = A_S(jj);
        cinc(BF == 1 ? C_N_splitFg : C_N_splitBg);
        float u1 = urand();
        float u2, u3;
        if (!EXACT && K->proposal == BAMF_PROPOSAL_LEARNED && urand() < 0.5f) {
            /* learned split: the first emitter's position from the learned
             * density and the intensity fraction from a triangular density on
             * [0.3, 0.7] (the mixture density of (u1, offset) enters
             * finish_split) */
            float lx, ly;
            learned_position(&lx, &ly);
            u1 = 0.3f + 0.2f * (urand() + urand());
            u2 = lx - mux;
            u3 = ly - muy;
        } else {
            u2 = p.Split_std * randn();
            u3 = p.Split_std * randn();
        }
        setT(jj, u1 * Ijp, mux + u2, muy + u3);
        if (!EXACT) a_dirty |= 1u << jj;
        addT((1.0f - u1) * Ijp, mux - u1 * u2 / (1.0f - u1), muy - u1 * u3 / (1.0f - u1), BF);
        pk_move = MV_SPLIT;
        pk_type = 4;
        pk_i0 = jj;
        pk_f0 = u1;
        pk_f1 = u2;
        pk_f2 = u3;
        pk_f3 = Ijp;
        pk_c1 = C_A_split;
        pk_c2 = BF == 1 ? C_A_splitFg : C_A_splitBg;
        if (t_overflow) {
            overflow++;
            return ACT_REJECT;
        }
        return testT() ? ACT_EVAL : ACT_REJECT;
    }
    __device__ __forceinline__ float finish_split(float LLR)
    {
        const bamf_mcmc_params &p = K->p;
        int jj = pk_i0;
        float u1 = pk_f0, u2 = pk_f1, u3 = pk_f2, Ijp = pk_f3;
        float tmp1 = 1.0f, tmp2 = 1.0f;
        tmp1 = tmp1 * sob(A_S(jj), A_I(jj));
        tmp2 = tmp2 * sob(T_S(jj), T_I(jj));
        tmp2 = tmp2 * sob(T_S(tn - 1), T_I(tn - 1));
        float Norm1 = normpdf(u2, 0.0f, p.Split_std);
        float Norm2 = normpdf(u3, 0.0f, p.Split_std);
        float NEm = nsignalA();
        float PrM = MeanN / (NEm + 1.0f);
        float PrI = tmp2 / tmp1;
        float Area = (float)(((float)X + p.Bnd_out) * ((float)Y + p.Bnd_out));
        float PrX = 1.0f / Area;
        float Us = 1.0f / (Norm1 * Norm2);
        float om = 1.0f - u1;
        float Jacob = EXACT ? (float)(__ddiv_rn((double)Ijp, dmul((double)om, (double)om))) : Ijp / (om * om);
        if (!EXACT && K->proposal != BAMF_PROPOSAL_REFERENCE) {
            /* exact split/merge pair accounting: the merge proposes this pair
             * with probability (1/k_a + 1/k_b) / (n + 1) (a random partner
             * within 3 sigma of a random emitter; k = such partners), the
             * split draws it from either emitter as the first:
             * (1/n) (q_a / J_a + q_b / J_b) */
            const float xa = __shfl_sync(BAMF_FULL, tX, jj), ya = __shfl_sync(BAMF_FULL, tY, jj);
            const float xb = __shfl_sync(BAMF_FULL, tX, tn - 1), yb = __shfl_sync(BAMF_FULL, tY, tn - 1);
            const float dmax = 3.0f * sigma;
            const float dx = xa - xb, dy = ya - yb;
            if (!(sqrtf(dx * dx + dy * dy) < dmax)) return 0.0f; /* no merge undoes it */
            const float ka = (float)near_count_T(jj, dmax), kb = (float)near_count_T(tn - 1, dmax);
            const float mux = A_X(jj), muy = A_Y(jj);
            const float qa = pair_density(u1, xa - mux, ya - muy, xa, ya, Ijp);
            const float qb = pair_density(1.0f - u1, xb - mux, yb - muy, xb, yb, Ijp);
            return LLR * PrI * (1.0f / box_area()) * (P[2] / P[1]) * PrM * (float)an * (1.0f / ka + 1.0f / kb) /
                   (qa + qb);
        }
        return LLR * PrI * PrX * Us * Jacob * (P[1] / P[2]) * PrM;
    }

    /* RJMCMC::merge (:1111-1255). */
    __device__ __forceinline__ int propose_merge()
    {
        cinc(C_N_merge);
        copyA2T();
        if (an < 2) return ACT_GRIDS;
        float Ua = urand();
        int jj = min((int)floorf((float)an * Ua), an - 1);
        int ii = closest(jj, 3 * sigma);
        int aSj = A_S(jj);
        cinc(aSj == 1 ? C_N_mergeFg : C_N_mergeBg);
        float aIj = A_I(jj), aXj = A_X(jj), aYj = A_Y(jj);
        float aIi = A_I(ii), aXi = A_X(ii), aYi = A_Y(ii);
        {
            float dx = aXj - aXi, dy = aYj - aYi;
            float d2 = EXACT ? (float)dadd(dmul((double)dx, (double)dx), dmul((double)dy, (double)dy))
                             : dx * dx + dy * dy;
            if (sqrtf(d2) > 3 * sigma) return ACT_GRIDS;
        }
        float Ijp = aIj + aIi;
        float muxjp = (aIj * aXj + aIi * aXi) / Ijp;
        float muyjp = (aIj * aYj + aIi * aYi) / Ijp;
        float u1 = aIj / Ijp;
        float u2 = aXj - muxjp;
        float u3 = aYj - muyjp;
        setT(jj, Ijp, muxjp, muyjp);
        float PDFfg = findPDF(K->sig, Ijp);
        float PDFbg = findPDF(K->back, Ijp);
        if (lane == jj) tS = (PDFbg > PDFfg) ? 0 : 1;
        if (!EXACT) a_dirty |= (1u << jj) | (1u << ii);
        removeT(ii);
        pk_move = MV_MERGE;
        pk_type = 5;
        pk_i0 = jj;
        pk_i1 = ii;
        pk_i2 = aSj;
        pk_f0 = u1;
        pk_f1 = u2;
        pk_f2 = u3;
        pk_f3 = Ijp;
        pk_f4 = aIj;
        pk_f5 = aIi;
        pk_c1 = aSj == 1 ? C_A_mergeFg : C_A_mergeBg;
        pk_c2 = C_A_merge;
        return testT() ? ACT_EVAL : ACT_REJECT;
    }
    __device__ __forceinline__ float finish_merge(float LLR)
    {
        const bamf_mcmc_params &p = K->p;
        int jj = pk_i0, ii = pk_i1, aSj = pk_i2;
        float u1 = pk_f0, u2 = pk_f1, u3 = pk_f2, Ijp = pk_f3, aIj = pk_f4, aIi = pk_f5;
        float tmp1 = 1.0f, tmp2 = 1.0f;
        tmp1 = tmp1 * sob(aSj, aIj);
        tmp1 = tmp1 * sob(A_S(ii), aIi);
        int jt = ii > jj ? jj : jj - 1;
        tmp2 = tmp2 * sob(T_S(jt), T_I(jt));
        float Norm1 = normpdf(u2, 0.0f, p.Split_std);
        float Norm2 = normpdf(u3, 0.0f, p.Split_std);
        float NEm = nsignalA();
        float PrI = tmp1 / tmp2;
        float Area = (float)(((float)X + p.Bnd_out) * ((float)Y + p.Bnd_out));
        float PrX = 1.0f / Area;
        float Us = 1.0f / (Norm1 * Norm2);
        float om = 1.0f - u1;
        float Jacob = EXACT ? (float)(__ddiv_rn((double)Ijp, dmul((double)om, (double)om))) : Ijp / (om * om);
        float PrM = MeanN / NEm;
        if (!EXACT && K->proposal != BAMF_PROPOSAL_REFERENCE) {
            /* the inverse of the split ratio that would undo this merge
             * (pair accounting as in finish_split) */
            const float dmax = 3.0f * sigma;
            const float kj = (float)__popc(near_mask(jj, dmax)), ki = (float)__popc(near_mask(ii, dmax));
            const float muxjp = __shfl_sync(BAMF_FULL, tX, jj > ii ? jj - 1 : jj);
            const float muyjp = __shfl_sync(BAMF_FULL, tY, jj > ii ? jj - 1 : jj);
            const float xa = A_X(jj), ya = A_Y(jj), xb = A_X(ii), yb = A_Y(ii);
            const float qa = pair_density(u1, xa - muxjp, ya - muyjp, xa, ya, Ijp);
            const float qb = pair_density(1.0f - u1, xb - muxjp, yb - muyjp, xb, yb, Ijp);
            return LLR / (PrI * (1.0f / box_area()) * (P[2] / P[1]) * PrM * (float)(an - 1) *
                          (1.0f / kj + 1.0f / ki) / (qa + qb));
        }
        return LLR / (PrI * PrX * Jacob * Us * PrM * P[1] / P[2]);
    }

    /* Density of a split that makes (x1, y1) the first emitter, over the
     * Jacobian: q(u1, u) (1 - u1)^2 / I for intensity fraction u1 and offset
     * u = (first emitter) - (split emitter).  q: UNIFORM, U(0, 1) x
     * N(0, Split_std^2)^2; LEARNED, half of that and half the triangular
     * density on [0.3, 0.7] x the learned density at (x1, y1). */
    __device__ __forceinline__ float pair_density(float u1, float u2, float u3, float x1, float y1, float I) const
    {
        const float s = K->p.Split_std;
        float q = normpdf(u2, 0.0f, s) * normpdf(u3, 0.0f, s);
        if (K->proposal == BAMF_PROPOSAL_LEARNED) {
            const int64_t off = B->offsets[roi];
            const float ql = learned_density(x1, y1, X, Y, npix, B->birth_cdf + off, B->birth_sub + 16 * off);
            const float tri = fmaxf(0.0f, 1.0f - fabsf(u1 - 0.5f) * 5.0f) * 5.0f;
            q = 0.5f * q + 0.5f * tri * ql;
        }
        const float om = 1.0f - u1;
        return q * om * om / I;
    }
    /* emitters of T within dmin of T's emitter k (k excluded) */
    __device__ __forceinline__ int near_count_T(int k, float dmin) const
    {
        const float xk = __shfl_sync(BAMF_FULL, tX, k), yk = __shfl_sync(BAMF_FULL, tY, k);
        const float dx = tX - xk, dy = tY - yk;
        return __popc(__ballot_sync(BAMF_FULL, lane < tn && lane != k && sqrtf(dx * dx + dy * dy) < dmin));
    }

    /* Area of the extended box [-Bnd, X+Bnd] x [-Bnd, Y+Bnd] that test()
     * admits (Bnd = (int)Bnd_out): the support of the position prior. */
    __device__ __forceinline__ float box_area() const
    {
        int bnd = (int)K->p.Bnd_out;
        return (float)(X + 2 * bnd) * (float)(Y + 2 * bnd);
    }

    /* Birth position of the UNIFORM and LEARNED proposals: uniform on the
     * extended box, or (LEARNED, with probability 1/2) a pixel drawn from
     * the ROI's running sum birth_cdf, a sub-cell drawn from birth_sub and a
     * uniform point inside that sub-cell. */
    __device__ __forceinline__ void birth_position(float *bx, float *by)
    {
        const int bnd = (int)K->p.Bnd_out;
        bool learned = K->proposal == BAMF_PROPOSAL_LEARNED && urand() < 0.5f;
        if (!learned) {
            *bx = (float)(-bnd) + (float)(X + 2 * bnd) * urand();
            *by = (float)(-bnd) + (float)(Y + 2 * bnd) * urand();
            return;
        }
        learned_position(bx, by);
    }

    /* A position drawn from the learned density: a pixel from the ROI's
     * running sum birth_cdf, a sub-cell from birth_sub, a uniform point in
     * the sub-cell.  Call with the whole warp. */
    __device__ __forceinline__ void learned_position(float *bx, float *by)
    {
        const int64_t off = B->offsets[roi];
        const float *cdf = B->birth_cdf + off;
        float rr = urand() * __ldg(&cdf[npix - 1]);
        /* the first pixel whose running sum reaches rr, in two rounds of
         * loads: the first 32-pixel block whose last sum reaches it (npix <=
         * 1024, so one lane per block), then the pixel inside it */
        const int nblk = (npix + 31) >> 5;
        const uint32_t mb =
            __ballot_sync(BAMF_FULL, lane < nblk && rr <= __ldg(&cdf[min(32 * lane + 31, npix - 1)]));
        const int blk = mb ? __ffs(mb) - 1 : nblk - 1;
        const int q = 32 * blk + lane;
        const uint32_t mp = __ballot_sync(BAMF_FULL, q < npix && rr <= __ldg(&cdf[min(q, npix - 1)]));
        const int pix = mp ? 32 * blk + __ffs(mp) - 1 : npix - 1;
        const float *sub = B->birth_sub + 16 * (off + pix);
        float v = lane < 16 ? __ldg(&sub[lane]) : 0.0f;
        for (int o = 1; o < 16; o <<= 1) {
            float t = __shfl_up_sync(BAMF_FULL, v, o);
            if (lane >= o) v += t;
        }
        float tot = __shfl_sync(BAMF_FULL, v, 15);
        float r2 = urand() * tot;
        uint32_t m = __ballot_sync(BAMF_FULL, lane < 16 && r2 <= v);
        int sc = m ? __ffs(m) - 1 : 15;
        int px = pix / Y, py = pix - px * Y;
        *bx = (float)px + ((float)(sc >> 2) + urand()) * 0.25f;
        *by = (float)py + ((float)(sc & 3) + urand()) * 0.25f;
    }

    /* (1 / box area) / q(x, y): the position prior over the birth proposal
     * density at (x, y); 1 for UNIFORM. */
    __device__ __forceinline__ float birth_q_ratio(float x, float y) const
    {
        if (K->proposal != BAMF_PROPOSAL_LEARNED) return 1.0f;
        const int64_t off = B->offsets[roi];
        return learned_q_ratio(x, y, X, Y, npix, box_area(), B->birth_cdf + off, B->birth_sub + 16 * off);
    }

    /* RJMCMC::find_Birth (:1688-1736); PixProb is overwritten with 1. */
    __device__ __forceinline__ void find_birth(float *bx, float *by)
    {
        float total;
        float *Pf = EXACT ? E : Mt; /* prefix buffer; Mt is free before the proposal is scored */
        if (EXACT) {
            for (int p = lane; p < npix; p += 32) {
                float v = D[p] - M[p];
                E[p] = (0.0f > v) ? 0.0f : v;
            }
            __syncwarp();
            if (lane == 0)
                for (int p = 1; p < npix; ++p) E[p] += E[p - 1];
            __syncwarp();
            total = E[npix - 1];
        } else {
            /* Fast: the residual's running sum is never stored.  Lane j sums
             * the contiguous chunk j of ceil(npix/32) pixels, a warp scan
             * gives the chunk ends, a ballot finds the chunk that reaches
             * rr, and that chunk's pixels (one per lane) are scanned again
             * to find the pixel: the same draw (the first pixel whose
             * running sum reaches rr), two passes over the chunk's pixels
             * instead of three over all. */
            const int per = (npix + 31) >> 5;
            const int p0 = min(lane * per, npix), p1 = min(p0 + per, npix);
            float s = 0.0f;
#pragma unroll 1
            for (int p = p0; p < p1; ++p) {
                float v = D[p] - M[p];
                s += v > 0.0f ? v : 0.0f;
            }
            float incl = s;
            for (int o = 1; o < 32; o <<= 1) {
                float t = __shfl_up_sync(BAMF_FULL, incl, o);
                if (lane >= o) incl += t;
            }
            total = __shfl_sync(BAMF_FULL, incl, 31);
            const float rr = total * urand();
            const uint32_t mc = __ballot_sync(BAMF_FULL, p0 < p1 && rr <= incl);
            int ii;
            if (mc) {
                const int cj = __ffs(mc) - 1;
                const float base = __shfl_sync(BAMF_FULL, incl - s, cj);
                const int q0 = cj * per, q = q0 + lane;
                float v = 0.0f;
                if (lane < per && q < npix) {
                    v = D[q] - M[q];
                    v = v > 0.0f ? v : 0.0f;
                }
                for (int o = 1; o < 32; o <<= 1) {
                    float t = __shfl_up_sync(BAMF_FULL, v, o);
                    if (lane >= o) v += t;
                }
                const uint32_t mq = __ballot_sync(BAMF_FULL, lane < per && q < npix && rr <= base + v);
                ii = mq ? q0 + __ffs(mq) - 1 : min(q0 + per, npix) - 1;
            } else {
                ii = npix; /* rr beyond the total (total 0: every pixel zero) */
            }
            *by = (float)(ii - Y * (ii / Y)) + urand() - 0.5f;
            *bx = (float)(int)floorf((float)ii / (float)Y) + urand() - 0.5f;
            return;
        }
        float rr = total * urand();
        int first = npix;
#pragma unroll 1
        for (int p = lane; p < npix; p += 32)
            if (rr <= Pf[p]) {
                first = p;
                break;
            }
        for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(BAMF_FULL, first, o));
        int ii = first;
        *by = (float)(ii - Y * (ii / Y)) + urand() - 0.5f;
        *bx = (float)(int)floorf((float)ii / (float)Y) + urand() - 0.5f;
        __syncwarp();
    }

    /* RJMCMC::birth (:1258-1330). */
    __device__ __forceinline__ int propose_birth()
    {
        cinc(C_N_birth);
        copyA2T();
        const bamf_mcmc_params &p = K->p;
        float bx, by;
        if (!EXACT && K->proposal != BAMF_PROPOSAL_REFERENCE) birth_position(&bx, &by);
        else find_birth(&bx, &by);
        pk_f0 = bx;
        pk_f1 = by;
        int BF;
        if (p.IsBackg == 1) BF = EXACT ? (int)floor(dadd((double)urand(), 0.5)) : (int)floorf(urand() + 0.5f);
        else BF = 1;
        float I_new;
        if (BF == 1) {
            cinc(C_N_birthFg);
            I_new = genRand(K->sig);
        } else {
            cinc(C_N_birthBg);
            I_new = genRand(K->back);
        }
        addT(I_new, bx, by, BF);
        pk_move = MV_BIRTH;
        pk_type = 6;
        pk_c1 = BF == 1 ? C_A_birthFg : C_A_birthBg;
        pk_c2 = C_A_birth;
        if (t_overflow) {
            overflow++;
            return ACT_REJECT;
        }
        return testT() ? ACT_EVAL : ACT_REJECT;
    }
    __device__ __forceinline__ float finish_birth(float LLR)
    {
        const bamf_mcmc_params &p = K->p;
        float NEm = nsignalA();
        float PrM = MeanN / (NEm + 1.0f);
        if (!EXACT && K->proposal != BAMF_PROPOSAL_REFERENCE)
            return LLR * PrM * (P[4] / P[3]) * birth_q_ratio(pk_f0, pk_f1);
        const float PixProb = 1.0f;
        return LLR * P[3] / (P[4] * ((float)X + p.Bnd_out) * ((float)Y + p.Bnd_out) * PixProb) * PrM;
    }

    /* RJMCMC::death (:1332-1387). */
    __device__ __forceinline__ int propose_death()
    {
        cinc(C_N_death);
        copyA2T();
        if (an < 1) return ACT_SKIP;
        float Ua = urand();
        int jj = min((int)floorf((float)an * Ua), an - 1);
        int aSj = A_S(jj);
        cinc(aSj == 1 ? C_N_deathFg : C_N_deathBg);
        if (!EXACT) a_dirty |= 1u << jj;
        removeT(jj);
        pk_move = MV_DEATH;
        pk_type = 7;
        pk_i0 = jj;
        pk_c1 = C_A_death;
        pk_c2 = aSj == 1 ? C_A_deathFg : C_A_deathBg;
        return ACT_EVAL;
    }
    __device__ __forceinline__ float finish_death(float LLR)
    {
        float NEm = nsignalA();
        float PrM = NEm / MeanN;
        if (!EXACT && K->proposal != BAMF_PROPOSAL_REFERENCE)
            return LLR * PrM * (P[3] / P[4]) / birth_q_ratio(A_X(pk_i0), A_Y(pk_i0));
        return LLR * (P[4] / P[3]) * PrM;
    }

    /* RJMCMC::gSplit (:1389-1485).  The reference does not test the
     * proposal's bounds here. */
    __device__ __forceinline__ int propose_gsplit()
    {
        if (an < 2) return ACT_SKIP;
        copyA2T();
        float Ua = urand();
        int jj = min((int)floorf((float)an * Ua), an - 1);
        int Np = closestMulti(jj, 2 * sigma);
        if (lane == 0) cl[Np] = jj;
        __syncwarp();
        Np++;
        if (Np == 1) return ACT_SKIP;
        float I0 = 0.0f, X0 = 0.0f, Y0 = 0.0f;
        for (int n = 0; n < Np; ++n) {
            int c = cl[n];
            I0 = I0 + A_I(c);
            X0 = X0 + A_X(c);
            Y0 = Y0 + A_Y(c);
        }
        float u1 = 0.3f * randn();
        float u2 = 0.3f * randn();
        float u3 = (1.0f / (float)Np) * urand();
        for (int n = 0; n < Np; ++n) {
            int c = cl[n];
            float aXc = A_X(c), aYc = A_Y(c), aIc = A_I(c);
            setT(c, (1.0f - u3) * aIc, (aXc - u3 * (X0 / (float)Np + u1)) / (1.0f - u3),
                 (aYc - u3 * (Y0 / (float)Np + u2)) / (1.0f - u3));
            if (!EXACT) a_dirty |= 1u << c;
        }
        addT(u3 * I0, X0 / (float)Np + u1, Y0 / (float)Np + u2, 1);
        pk_move = MV_GSPLIT;
        pk_type = 8;
        pk_i0 = Np;
        pk_f0 = u1;
        pk_f1 = u2;
        pk_f2 = u3;
        pk_f3 = I0;
        pk_c1 = pk_c2 = -1;
        if (t_overflow) {
            overflow++;
            return ACT_REJECT;
        }
        return ACT_EVAL;
    }
    __device__ __forceinline__ float finish_gsplit(float LLR)
    {
        int Np = pk_i0;
        float u1 = pk_f0, u2 = pk_f1, u3 = pk_f2, I0 = pk_f3;
        float PrI = 1.0f, tmpCurrent, tmpProposed;
        for (int n = 0; n < Np; ++n) {
            int c = cl[n];
            tmpCurrent = sob(A_S(c), A_I(c));
            tmpProposed = sob(T_S(n), T_I(c));
            PrI = PrI * tmpProposed / tmpCurrent;
        }
        tmpProposed = sob(T_S(tn - 1), T_I(tn - 1));
        PrI = PrI * (tmpProposed);
        float PDFu1 = normpdf(u1, 0.0f, 0.4f);
        float PDFu2 = normpdf(u2, 0.0f, 0.4f);
        float PDFu3 = (float)Np;
        float Us = 1.0f / (PDFu1 * PDFu2 * PDFu3);
        float NEm = nsignalA();
        float PrM = MeanN / (NEm + 1.0f);
        const bamf_mcmc_params &p = K->p;
        float Area = (float)(((float)X + p.Bnd_out) * ((float)Y + p.Bnd_out));
        float PrX = 1.0f / Area;
        float Jacob = I0 / MT::powf_(1.0f - u3, (float)(Np + 1));
        return LLR * PrI * PrX * Us * Jacob * PrM * (P[5] / P[6]);
    }

    /* RJMCMC::gMerge (:1487-1584). */
    __device__ __forceinline__ int propose_gmerge()
    {
        if (an < 3) return ACT_SKIP;
        copyA2T();
        float Ua = urand();
        int jj = min((int)floorf((float)an * Ua), an - 1);
        int Np = closestMulti(jj, 3 * sigma);
        if (Np == 0) return ACT_SKIP;
        float aIj = A_I(jj), aXj = A_X(jj), aYj = A_Y(jj);
        float I0 = aIj;
        for (int n = 0; n < Np; ++n) I0 = I0 + A_I(cl[n]);
        float XX0 = 0.0f, YY0 = 0.0f;
        float U3 = aIj / I0;
        for (int n = 0; n < Np; ++n) {
            int c = cl[n];
            float aIc = A_I(c), aXc = A_X(c), aYc = A_Y(c);
            float nX = U3 * aXj + (1.0f - U3) * aXc;
            XX0 = XX0 + U3 * aXj + (1.0f - U3) * aXc;
            float nY = U3 * aYj + (1.0f - U3) * aYc;
            YY0 = YY0 + U3 * aYj + (1.0f - U3) * aYc;
            setT(c, aIc / (1.0f - U3), nX, nY);
            if (!EXACT) a_dirty |= 1u << c;
        }
        float U1 = aXj - XX0 / (float)Np;
        float U2 = aYj - YY0 / (float)Np;
        float PrI = 1.0f, tmpProposed, tmpCurrent;
        for (int n = 0; n < Np; ++n) {
            int c = cl[n];
            tmpProposed = sob(T_S(c), T_I(c));
            tmpCurrent = sob(A_S(c), A_I(c));
            PrI = PrI * (tmpCurrent / tmpProposed);
        }
        tmpCurrent = sob(A_S(jj), aIj);
        PrI = PrI * tmpCurrent;
        if (!EXACT) a_dirty |= 1u << jj;
        removeT(jj);
        pk_move = MV_GMERGE;
        pk_type = 9;
        pk_i0 = Np;
        pk_f0 = U1;
        pk_f1 = U2;
        pk_f2 = U3;
        pk_f3 = I0;
        pk_f4 = PrI;
        pk_c1 = pk_c2 = -1;
        return ACT_EVAL;
    }
    __device__ __forceinline__ float finish_gmerge(float LLR)
    {
        int Np = pk_i0;
        float U1 = pk_f0, U2 = pk_f1, U3 = pk_f2, I0 = pk_f3, PrI = pk_f4;
        float PDFu1 = normpdf(U1, 0.0f, 0.4f);
        float PDFu2 = normpdf(U2, 0.0f, 0.4f);
        float PDFu3 = (float)Np;
        float Us = 1.0f / (PDFu1 * PDFu2 * PDFu3);
        float NEm = nsignalA();
        float PrM = NEm / MeanN;
        const bamf_mcmc_params &p = K->p;
        float Area = (float)(((float)X + p.Bnd_out) * ((float)Y + p.Bnd_out));
        float PrX = 1.0f / Area;
        float Jacob = I0 / MT::powf_(1.0f - U3, (float)(Np + 1));
        float PR = LLR / (PrI * PrX * Us * Jacob * PrM * (P[5] / P[6]));
        if (PDFu1 == 0.0f || PDFu2 == 0.0f) PR = -1.0f;
        return PR;
    }

    /* RJMCMC::backFore (:1586-1627): relabels in place, records nothing. */
    __device__ __forceinline__ void mv_backfore()
    {
        if (an == 0) return;
        if (K->p.IsBackg == 0) return;
        float Ua = urand();
        int nn = min((int)floorf((float)an * Ua), an - 1);
        float In = A_I(nn);
        int Sn = A_S(nn);
        float BackP = findPDF(K->back, In);
        float SignalP = findPDF(K->sig, In);
        int ns = Sn;
        if (Sn == 1) {
            if (SignalP != 0.0f) {
                float PrSig = BackP / SignalP;
                if (PrSig > urand()) ns = 0;
            } else {
                ns = 0;
            }
        } else {
            if (BackP != 0.0f) {
                float PrSig = SignalP / BackP;
                if (PrSig > urand()) ns = 1;
            } else {
                ns = 1;
            }
        }
        if (lane == nn) aS = ns;
    }

    /* One jump of start_Chain (:693-717, :725-748): W = this phase's
     * cumulative probabilities, V = PV_Burnin for the gSplit/gMerge slots. */
    __device__ __forceinline__ void step(const float *V, const float *W, float t)
    {
        int act;
        if (t < W[0]) act = propose_jump();
        else if (t >= W[0] && t < W[1]) act = propose_split();
        else if (t >= W[1] && t < W[2]) act = propose_merge();
        else if (t >= W[2] && t < W[3]) act = propose_birth();
        else if (t >= W[3] && t < W[4]) act = propose_death();
        else if (t >= V[4] && t < V[5]) act = propose_gsplit();
        else if (t >= V[5] && t < V[6]) act = propose_gmerge();
        else {
            mv_backfore();
            act = ACT_SKIP;
        }
        float LLR = 0.0f, PR = 0.0f;
        int accept = 0;
        if (act == ACT_EVAL) {
            LLR = llr();
            switch (pk_move) {
            case MV_JUMP: PR = finish_jump(LLR); break;
            case MV_SPLIT: PR = finish_split(LLR); break;
            case MV_MERGE: PR = finish_merge(LLR); break;
            case MV_BIRTH: PR = finish_birth(LLR); break;
            case MV_DEATH: PR = finish_death(LLR); break;
            case MV_GSPLIT: PR = finish_gsplit(LLR); break;
            default: PR = finish_gmerge(LLR); break;
            }
            accept = (urand() < PR);
            if (accept) {
                if (pk_c1 >= 0) cinc(pk_c1);
                if (pk_c2 >= 0) cinc(pk_c2);
                accept_T();
            }
        }
        if (act >= ACT_REJECT) record2(LLR, PR, pk_type, accept);
        if (act >= ACT_GRIDS) update_grids();
    }

    /* RJMCMC::start_Chain (:685-750). */
    /* Move-synchronous chain (fast mode): every warp of the CTA takes the
     * same move type and jump sub-branch at each jump, drawn from a stream
     * shared by the CTA, and the warps meet at a barrier before each jump,
     * so the warps of an SM run the same code.  For each chain the move
     * choice is still i.i.d. with the configured probabilities and
     * independent of its state, so its transition kernel is unchanged.
     * Warps without a ROI (the tail of the queue) only take the barriers. */
    __device__ __forceinline__ void run_chain_sync(bool active, uint32_t grp)
    {
        const bamf_mcmc_params &p = K->p;
        use_shared_ub = true;
        int since_rebuild = 0;
        const int total = p.N_Burnin + p.N_Trials;
        for (int n = 0; n < total; ++n) {
            __syncthreads();
            if (n == 0 || n == p.N_Burnin) {
                is_burnin = n < p.N_Burnin;
                /* the reference's ratios see the cumulative trial vector
                 * (LibRJMCMC.cpp:721-722); the other proposals use the raw one */
                const float *Pt = K->proposal == BAMF_PROPOSAL_REFERENCE ? K->PVT : p.P_Trials;
                for (int k = 0; k < 8; ++k) P[k] = is_burnin ? p.P_Burnin[k] : Pt[k];
            }
            if (!active) continue;
            float t = shared_uniform(K->seed, grp, (uint32_t)n, 0u);
            shared_ub = shared_uniform(K->seed, grp, (uint32_t)n, 1u);
            step(K->PVB, is_burnin ? K->PVB : K->PVT, t);
            if (++since_rebuild == 512) {
                rebuild_model();
                since_rebuild = 0;
            }
        }
    }

    __device__ __forceinline__ void run_chain()
    {
        const bamf_mcmc_params &p = K->p;
        is_burnin = 1;
        for (int k = 0; k < 8; ++k) P[k] = p.P_Burnin[k];
        int since_rebuild = 0;
        for (int n = 0; n < p.N_Burnin; ++n) {
            float t = urand();
            step(K->PVB, K->PVB, t);
            if (!EXACT && ++since_rebuild == 512) {
                rebuild_model();
                since_rebuild = 0;
            }
        }
        is_burnin = 0;
        for (int k = 0; k < 8; ++k) P[k] = K->PVT[k];
        for (int n = 0; n < p.N_Trials; ++n) {
            float t = urand();
            step(K->PVB, K->PVT, t);
            if (!EXACT && ++since_rebuild == 512) {
                rebuild_model();
                since_rebuild = 0;
            }
        }
    }
};

/* Loads ROI `roi` into a warp's carve-out and sets up its chain (the
 * set-up of cRJMCMC.cpp:103-148).  Returns false, with the ROI's status set,
 * when the ROI does not fit the launch. */
template <bool EXACT, bool NUM>
__device__ __forceinline__ bool begin_roi(ChainWarp<EXACT, NUM> &w, const SamplerConsts *Kp, const SamplerBatch &Bt,
                                          float *sw, int roi)
{
    const int lane = w.lane;
    w.roi = roi;
    int X = Bt.xsize[roi], Y = Bt.ysize[roi];
    w.X = X;
    w.Y = Y;
    w.npix = X * Y;
    w.px_dx = 32 / Y;
    w.px_dy = 32 - (32 / Y) * Y;
    int npix_max = Bt.side_max * Bt.side_max;
    int nxs = BAMF_NMAX * Bt.side_max;
    w.D = sw;
    w.M = sw + npix_max;
    w.Mt = sw + 2 * npix_max;
    float *scm_smem = nullptr;
    if (EXACT) {
        w.E = sw + 3 * npix_max;
        scm_smem = sw + 4 * npix_max;
        w.NX = sw + 5 * npix_max;
        w.NY = w.NX + nxs;
        w.NXt = w.NY + nxs;
        w.NYt = w.NXt + nxs;
        w.SXo = w.SYo = w.SXn = w.SYn = nullptr;
        w.cnt = (int *)(w.NYt + nxs);
    } else {
        const int rs = FAST_ROWS * Bt.side_max;
        w.E = nullptr;
        w.NX = w.NY = w.NXt = w.NYt = nullptr;
        w.SXo = sw + 3 * npix_max;
        w.SYo = w.SXo + rs;
        w.SXn = w.SYo + rs;
        w.SYn = w.SXn + rs;
        w.cnt = (int *)(w.SYn + rs);
    }
    w.cl = w.cnt + C_COUNT;
    int n0 = Bt.init_n ? Bt.init_n[roi] : 0;
    bool ok = X >= 1 && Y >= 1 && X <= Bt.side_max && Y <= Bt.side_max && n0 <= BAMF_NMAX;
    if (!ok) {
        if (lane == 0 && Bt.status) Bt.status[roi] = BAMF_ERR_TOO_LARGE;
        return false;
    }
    const float *src = Bt.data + Bt.offsets[roi];
    const float *scm_src = Bt.scmos ? Bt.scmos + Bt.offsets[roi] : nullptr;
    for (int p = lane; p < w.npix; p += 32) {
        w.D[p] = src[p];
        if (EXACT) scm_smem[p] = scm_src ? scm_src[p] : 0.0f;
    }
    w.scm = EXACT ? scm_smem : scm_src;
    if (lane < C_COUNT) {
        int k = lane;
        bool isN = (k <= C_N_death) || (k >= C_N_jumpFg && k <= C_N_deathFg) ||
                   (k >= C_N_jumpBg && k <= C_N_deathBg);
        w.cnt[k] = isN ? 1 : 0;
    }
    float s = Bt.psf_sigma ? Bt.psf_sigma[roi] : Kp->p.PSFsigma;
    w.sigma = s;
    w.Cst = 1.0f / (s * sqrtf(2.0f));
    if (NUM) {
        const int32_t *P = Kp->p.PSFsize;
        w.pn0 = P[0];
        w.pn01 = P[0] * P[1];
        w.pn012 = w.pn01 * P[2];
        w.ptot = w.pn012 * P[3];
        w.pos = P[3];
        const int slot = Bt.psf_slot ? Bt.psf_slot[roi] : 0;
        if (slot < 0 || slot >= Bt.n_psf) {
            if (lane == 0 && Bt.status) Bt.status[roi] = BAMF_ERR_INVALID_ARG;
            return false;
        }
        w.psf = Bt.sampled_psf + (int64_t)slot * w.ptot;
    } else {
        w.psf = nullptr;
    }
    w.MeanN = Kp->p.Rho * (float)X * (float)Y;
    /* start state (cRJMCMC.cpp:120-133) */
    w.an = n0;
    w.aI = w.aX = w.aY = 0.0f;
    w.aS = 1;
    if (n0 > 0 && lane < n0) {
        const float *ixy = Bt.init_ixy + (size_t)roi * 3 * BAMF_NMAX;
        w.aI = ixy[lane];
        w.aX = ixy[BAMF_NMAX + lane];
        w.aY = ixy[2 * BAMF_NMAX + lane];
    }
    w.aBG = Bt.init_bg ? Bt.init_bg[roi] : Kp->bg0;
    if (w.aBG == 0.0f) w.aBG = 1.0f;
    if (!EXACT) w.pdf_aBG = w.findPDF(Kp->off, w.aBG);
    w.aABG = 0.0f;
    w.aBBG = 0.0f;
    w.seed = Kp->seed;
    w.chain = Bt.chain_ids ? Bt.chain_ids[roi] : (uint32_t)roi;
    w.idx = Bt.rng_offset ? Bt.rng_offset[roi] : 0u;
    w.base = w.idx >> 2;
    w.refill();
    w.entries = 0;
    w.overflow = 0;
    w.n_llr = 0;
    w.a_dirty = w.t_dirty = 0u;
    w.use_shared_ub = false;
    w.shared_ub = 0.0f;
    w.rec_n[0] = w.rec_n[1] = 0;
    if (!EXACT && Bt.model_drift && lane == 0) Bt.model_drift[roi] = 0.0f;
    __syncwarp();
    w.rebuild_model();
    return true;
}

/* Writes the chain's per-ROI results. */
template <bool EXACT, bool NUM>
__device__ __forceinline__ void end_roi(ChainWarp<EXACT, NUM> &w, const SamplerBatch &Bt)
{
    const int lane = w.lane, roi = w.roi;
    if (Bt.final_n && lane == 0) Bt.final_n[roi] = w.an;
    if (Bt.final_state) {
        float *fs = Bt.final_state + (size_t)roi * (4 + 4 * BAMF_NMAX);
        if (lane == 0) {
            fs[0] = w.aBG; fs[1] = w.aABG; fs[2] = w.aBBG; fs[3] = (float)w.an;
        }
        fs[4 + lane] = lane < w.an ? w.aI : 0.0f;
        fs[4 + BAMF_NMAX + lane] = lane < w.an ? w.aX : 0.0f;
        fs[4 + 2 * BAMF_NMAX + lane] = lane < w.an ? w.aY : 0.0f;
        fs[4 + 3 * BAMF_NMAX + lane] = lane < w.an ? (float)w.aS : 0.0f;
    }
    __syncwarp();
    if (Bt.counters)
        for (int k = lane; k < C_COUNT; k += 32) Bt.counters[(size_t)roi * C_COUNT + k] = w.cnt[k];
    if (Bt.chains && lane == 0) {
        Bt.chains[2 * roi].n_entries = min(w.entries, Bt.chains[2 * roi].capacity_entries);
        Bt.chains[2 * roi + 1].n_entries = min(w.entries, Bt.chains[2 * roi + 1].capacity_entries);
        Bt.chains[2 * roi].n_records = w.rec_n[0];
        Bt.chains[2 * roi + 1].n_records = w.rec_n[1];
    }
    if (lane == 0) {
        if (Bt.n_entries) Bt.n_entries[roi] = w.entries;
        if (Bt.uniforms_used) Bt.uniforms_used[roi] = w.idx - (Bt.rng_offset ? Bt.rng_offset[roi] : 0u);
        if (Bt.overflow) Bt.overflow[roi] = w.overflow;
        if (Bt.llr_evals) Bt.llr_evals[roi] = w.n_llr;
        if (Bt.status) Bt.status[roi] = BAMF_OK;
    }
    __syncwarp();
}

/* Persistent sampler: each warp pulls ROI ids from the work queue and runs
 * their chains one after another. */
template <bool EXACT, bool NUM>
__global__ void __launch_bounds__(128, 4) rjmcmc_kernel(const __grid_constant__ SamplerConsts Kc,
                                                     const __grid_constant__ SamplerBatch Bc)
{
    extern __shared__ float smem_raw[];
    const SamplerBatch &Bt = Bc;
    int warp = threadIdx.x >> 5;
    int lane = threadIdx.x & 31;
    float *sw = smem_raw + (size_t)warp * warp_smem_floats(Bt.side_max, EXACT);
    ChainWarp<EXACT, NUM> w;
    w.K = &Kc;
    w.B = &Bc;
    w.lane = lane;
    int q_begin = 0, q_end = Bt.n_rois;
    if (Bt.class_range) {
        q_begin = Bt.class_range[2 * Bt.cls];
        q_end = Bt.class_range[2 * Bt.cls + 1];
    }
    for (;;) {
        int slot = 0;
        if (lane == 0) slot = q_begin + atomicAdd(Bt.queue, 1);
        slot = __shfl_sync(BAMF_FULL, slot, 0);
        if (slot >= q_end) break;
        int roi = Bt.order ? Bt.order[slot] : slot;
        if (!begin_roi(w, &Kc, Bt, sw, roi)) continue;
        w.run_chain();
        end_roi(w, Bt);
    }
}

/* Move-synchronous persistent sampler (fast arithmetic): the CTA pulls one
 * ROI per warp at a time and its warps run their chains in lockstep, one
 * barrier per jump, with the move type and jump sub-branch shared across the
 * CTA (run_chain_sync). */
template <bool NUM, int MIN_CTAS>
__global__ void __launch_bounds__(MIN_CTAS == 1 ? 32 * BAMF_SYNC_GROUP : 256, MIN_CTAS) rjmcmc_kernel_sync(const __grid_constant__ SamplerConsts Kc,
                                                          const __grid_constant__ SamplerBatch Bc)
{
    extern __shared__ float smem_raw[];
    __shared__ int grp_base;
    const SamplerBatch &Bt = Bc;
    const int nwarps = blockDim.x >> 5;
    int warp = threadIdx.x >> 5;
    int lane = threadIdx.x & 31;
    float *sw = smem_raw + (size_t)warp * warp_smem_floats(Bt.side_max, false);
    ChainWarp<false, NUM> w;
    w.K = &Kc;
    w.B = &Bc;
    w.lane = lane;
    int q_begin = 0, q_end = Bt.n_rois;
    if (Bt.class_range) {
        q_begin = Bt.class_range[2 * Bt.cls];
        q_end = Bt.class_range[2 * Bt.cls + 1];
    }
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) grp_base = q_begin + atomicAdd(Bt.queue, nwarps);
        __syncthreads();
        int base = grp_base;
        if (base >= q_end) break;
        int slot = base + warp;
        bool active = slot < q_end;
        if (active) {
            int roi = Bt.order ? Bt.order[slot] : slot;
            active = begin_roi(w, &Kc, Bt, sw, roi);
        }
        /* the shared move stream is keyed by the slot group of BAMF_SYNC_GROUP
         * ROIs, not by the CTA, so a chain's moves (and its result) do not
         * depend on the launch's warps per block (any divisor of the group) */
        w.run_chain_sync(active, (uint32_t)(q_begin + (base - q_begin) / BAMF_SYNC_GROUP * BAMF_SYNC_GROUP));
        if (active) end_roi(w, Bt);
    }
}

}  // namespace bamf
