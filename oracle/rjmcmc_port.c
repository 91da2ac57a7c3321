/*
 * rjmcmc_port.c - TEST INFRASTRUCTURE: a plain-C restatement of the
 * reference reversible-jump sampler (source/c/LibRJMCMC.cpp, class RJMCMC
 * and helpers; set-up from source/c/cRJMCMC.cpp).  Every float expression is
 * written in the reference's evaluation order and built with
 * -ffp-contract=off, so with the same uniform stream and the same math
 * functions it reproduces the reference chain bit for bit.
 *
 * Math: by default the project's parity erf/log/exp/pow
 * (include/bamf_parity_math.h); with -DBAMF_ORACLE_NATIVE_MATH glibc's
 * erff/logf/expf/powf, like the unmodified reference.
 *
 * Scope: both likelihood models of cRJMCMC.cpp:73-74: OptModel 0 (the
 * Gaussian PSF, Model/Stencil) and OptModel 1 (the sampled PSF, NumModel,
 * LibRJMCMC.cpp:67-170).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "bamf_parity_math.h"
#include "bamf_philox.h"
#include "oracle.h"

#ifdef BAMF_ORACLE_NATIVE_MATH
#define O_ERF(x) erff(x)
#define O_LOG(x) logf(x)
#define O_EXP(x) expf(x)
#define O_POWF(x, y) powf((x), (y))
#define O_POW2(x) ((double)(x) * (double)(x))
#else
#define O_ERF(x) bamf_pm_erff(x)
#define O_LOG(x) bamf_pm_logf(x)
#define O_EXP(x) bamf_pm_expf(x)
#define O_POWF(x, y) bamf_pm_powf((x), (y))
#define O_POW2(x) bamf_pm_pow_fi((x), 2)
#endif

#define REF_PI 3.141592 /* LibRJMCMCreturn.hpp:2 (a double literal) */

/* ---------------------------------------------------------------- vectors */
typedef struct { float *v; int n, cap; } fvec;
typedef struct { int32_t *v; int n, cap; } ivec;

static void fpush(fvec *a, float x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 256;
        a->v = (float *)realloc(a->v, (size_t)a->cap * sizeof(float));
    }
    a->v[a->n++] = x;
}

static void ipush(ivec *a, int32_t x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 256;
        a->v = (int32_t *)realloc(a->v, (size_t)a->cap * sizeof(int32_t));
    }
    a->v[a->n++] = x;
}

/* ------------------------------------------------------------ prior table */
/* Stat (LibRJMCMC.cpp:176-282). */
typedef struct {
    float *pdf, *x, *cdf, *ux, *uc;
    int L, nu;
} ostat;

static void stat_free(ostat *s)
{
    free(s->pdf); free(s->x); free(s->cdf); free(s->ux); free(s->uc);
    memset(s, 0, sizeof *s);
}

/* Stat::Stat (:176-217). */
static void stat_init(ostat *s, const float *in, float DX, int L)
{
    s->L = L;
    s->pdf = (float *)malloc((size_t)L * sizeof(float));
    s->x = (float *)malloc((size_t)L * sizeof(float));
    s->cdf = (float *)malloc((size_t)L * sizeof(float));
    s->ux = (float *)malloc((size_t)L * sizeof(float));
    s->uc = (float *)malloc((size_t)L * sizeof(float));
    float *xm = (float *)malloc((size_t)L * sizeof(float));
    s->cdf[0] = 0;
    s->x[0] = 0;
    xm[0] = 0;
    for (int i = 0; i < L; ++i) s->pdf[i] = in[i];
    for (int i = 1; i < L; ++i) {
        s->cdf[i] = s->cdf[i - 1] + (s->pdf[i] + s->pdf[i - 1]) * DX / 2.0f;
        if (s->cdf[i] > 1.0f) s->cdf[i] = 1.0f;
        xm[i] = s->cdf[i];
        s->x[i] = s->x[i - 1] + DX;
    }
    for (int i = L - 2; i >= 0; --i)
        if (s->cdf[i] == s->cdf[i + 1]) xm[i + 1] = -1;
    s->nu = 0;
    for (int i = 0; i < L; ++i) {
        if (xm[i] != -1) {
            s->ux[s->nu] = s->x[i];
            s->uc[s->nu] = s->cdf[i];
            s->nu++;
        }
    }
    if (s->uc[s->nu - 1] != 1) s->uc[s->nu - 1] = 1;
    if (s->uc[0] != 0) s->uc[0] = 0;
    free(xm);
}

/* Stat::findPDF (:219-246). */
static float stat_pdf(const ostat *s, float I, int *messages)
{
    int L = s->L;
    if (I >= s->x[L - 1] || I <= 0) return 0;
    int ind = -1;
    for (int j = 0; j < L; ++j) {
        if (s->x[j] - I > 0) {
            ind = j;
            break;
        }
    }
    if (ind == -1 || ind == 0) {
        ++*messages;
        return 0;
    }
    return (s->pdf[ind] * (I - s->x[ind - 1]) + s->pdf[ind - 1] * (s->x[ind] - I)) /
           (s->x[1] - s->x[0]);
}

/* ---------------------------------------------------------------- emitters */
typedef struct {
    int n, cap;
    float *I, *X, *Y;
    int *S;
    float BG, ABG, BBG;
} oem;

static void em_reserve(oem *e, int n)
{
    if (n <= e->cap) return;
    int c = e->cap ? e->cap : 16;
    while (c < n) c *= 2;
    e->I = (float *)realloc(e->I, (size_t)c * sizeof(float));
    e->X = (float *)realloc(e->X, (size_t)c * sizeof(float));
    e->Y = (float *)realloc(e->Y, (size_t)c * sizeof(float));
    e->S = (int *)realloc(e->S, (size_t)c * sizeof(int));
    e->cap = c;
}

static void em_free(oem *e)
{
    free(e->I); free(e->X); free(e->Y); free(e->S);
    memset(e, 0, sizeof *e);
}

static void em_copy(oem *d, const oem *s)
{
    em_reserve(d, s->n + 1);
    d->n = s->n;
    memcpy(d->I, s->I, (size_t)s->n * sizeof(float));
    memcpy(d->X, s->X, (size_t)s->n * sizeof(float));
    memcpy(d->Y, s->Y, (size_t)s->n * sizeof(float));
    memcpy(d->S, s->S, (size_t)s->n * sizeof(int));
    d->BG = s->BG; d->ABG = s->ABG; d->BBG = s->BBG;
}

/* Emitters::add (:470-476). */
static void em_add(oem *e, float I, float x, float y, int bf)
{
    em_reserve(e, e->n + 1);
    e->I[e->n] = I; e->X[e->n] = x; e->Y[e->n] = y; e->S[e->n] = bf;
    e->n++;
}

/* Emitters::remove (:478-490). */
static void em_remove(oem *e, int id)
{
    if (e->n == 0) return;
    for (int k = id; k < e->n - 1; ++k) {
        e->I[k] = e->I[k + 1]; e->X[k] = e->X[k + 1]; e->Y[k] = e->Y[k + 1]; e->S[k] = e->S[k + 1];
    }
    e->n--;
}

/* Emitters::test (:492-514); Bnd_out arrives cast to int. */
static int em_test(const oem *e, int bnd, int X, int Y)
{
    for (int n = 0; n < e->n; ++n) if (e->I[n] < 0) return 0;
    for (int n = 0; n < e->n; ++n) if (e->X[n] < (float)(-bnd)) return 0;
    for (int n = 0; n < e->n; ++n) if (e->Y[n] < (float)(-bnd)) return 0;
    for (int n = 0; n < e->n; ++n) if (e->X[n] > (float)(X + bnd)) return 0;
    for (int n = 0; n < e->n; ++n) if (e->Y[n] > (float)(Y + bnd)) return 0;
    return 1;
}

/* ------------------------------------------------------------------ chain */
typedef struct {
    ivec N, JumpType, Accepted, Index, Signal;
    fvec LLR, PR, BG, ABG, BBG, Photons, X, Y;
} ochain;

static void chain_free(ochain *c)
{
    free(c->N.v); free(c->JumpType.v); free(c->Accepted.v); free(c->Index.v); free(c->Signal.v);
    free(c->LLR.v); free(c->PR.v); free(c->BG.v); free(c->ABG.v); free(c->BBG.v);
    free(c->Photons.v); free(c->X.v); free(c->Y.v);
    memset(c, 0, sizeof *c);
}

/* ---------------------------------------------------------------- sampler */
typedef struct {
    int X, Y;
    const float *D;
    const float *scmos;
    bamf_mcmc_params p;
    float P[8], PVB[8], PVT[8];
    float MeanN;
    ostat off, sig, back;
    oem A, T;
    float *M, *Mt, *NX, *NY, *resid;
    int nx_cap;
    int is_burnin;
    uint32_t seed, chain, idx, blk_id;
    bamf_philox_block blk;
    int blk_valid;
    bamf_counters c;
    int record;      /* 1: full chain vectors; 0: only the N-signal trace */
    ochain ch[2];
    ivec nsig_trace; /* per accepted-chain entry: emitters with Signal == 1 */
    float *pgrid, *pback;
    int messages;
    int opt_model;     /* 0 Gaussian PSF, 1 sampled PSF */
    int first_call;    /* Params.FirstCall of the reference (see likelihood_ratio) */
    const float *psf;  /* [P0][P1][P2][P3] of p.PSFsize, first index fastest */
} orj;

static float urand(orj *r)
{
    uint32_t b = r->idx >> 2;
    if (!r->blk_valid || b != r->blk_id) {
        r->blk = bamf_philox4x32_10(b, 0u, 0u, 0u, r->seed, r->chain);
        r->blk_id = b;
        r->blk_valid = 1;
    }
    uint32_t k = r->blk.v[r->idx & 3u] >> 1;
    r->idx++;
    return bamf_u31_to_float(k);
}

/* randn: Irwin-Hall sum of 12 uniforms (LibRJMCMCreturn.hpp:23-26). */
static float randn(orj *r)
{
    float tmp = 0;
    for (int n = 0; n < 12; ++n) tmp = tmp + urand(r);
    return tmp - 6.0f;
}

/* normpdf (LibRJMCMCreturn.hpp:19-21). */
static float normpdf(float x, float u, float s)
{
    float d = x - u;
    return 1.0f / ((float)sqrt(2.0f * REF_PI) * s) * O_EXP(-d * d / (2 * s * s));
}

static int kround(float a) { return (int)floor((double)a + .5); }

static void ensure_stencil(orj *r, int n)
{
    if (n <= r->nx_cap) return;
    int c = r->nx_cap ? r->nx_cap : 16;
    while (c < n) c *= 2;
    r->NX = (float *)realloc(r->NX, (size_t)c * r->X * sizeof(float));
    r->NY = (float *)realloc(r->NY, (size_t)c * r->Y * sizeof(float));
    r->nx_cap = c;
}

/* Stencil (:15-36) + Model (:42-59). */
static void model(orj *r, const oem *E, float *M)
{
    int X = r->X, Y = r->Y;
    float C = 1 / (r->p.PSFsigma * sqrtf(2.0f));
    ensure_stencil(r, E->n);
    for (int n = 0; n < E->n; ++n)
        for (int x = 0; x < X; ++x)
            r->NX[X * n + x] = E->I[n] * 0.5f *
                               (O_ERF(((float)x - E->X[n] + 1.0f) * C) - O_ERF(((float)x - E->X[n]) * C));
    for (int n = 0; n < E->n; ++n)
        for (int y = 0; y < Y; ++y)
            r->NY[Y * n + y] =
                0.5f * (O_ERF(((float)y - E->Y[n] + 1.0f) * C) - O_ERF(((float)y - E->Y[n]) * C));
    for (int x = 0; x < X; ++x)
        for (int y = 0; y < Y; ++y)
            M[y + x * Y] = E->BG + E->ABG * x + E->BBG * y + r->scmos[x * Y + y];
    for (int n = 0; n < E->n; ++n)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x) M[y + x * Y] += r->NX[X * n + x] * r->NY[Y * n + y];
}

/* NumModel (:67-170).  The background plane, then per emitter, in order,
 * I times a bilinear blend of four samples of the PSF array: the emitter
 * sits on PSF pixel P0/2 (integer division), its fractional position picks
 * the sub-position planes ix = floor(P3 frac x) and ix + 1 (the next pixel's
 * plane 0 after the last), likewise in y, and the weights are the distance
 * to the next plane in units of 1/P3.  Positions and weights are computed
 * in double as there; the blend and the sum in float.  A flat index
 * outside the array reads the last element (one message each). */
static float psf_get(orj *r, int i, int total)
{
    if (i >= total || i < 0) {
        r->messages++;
        i = total - 1;
    }
    return r->psf[i];
}

static void num_model(orj *r, const oem *E, float *M)
{
    int X = r->X, Y = r->Y;
    const int32_t *P = r->p.PSFsize;
    const int s0 = P[0], s01 = P[0] * P[1], s012 = s01 * P[2], total = s012 * P[3];
    const double os = (double)P[3];
    const int c0 = P[0] / 2;
    for (int x = 0; x < X; ++x)
        for (int y = 0; y < Y; ++y)
            M[y + x * Y] = E->BG + E->ABG * x + E->BBG * y + r->scmos[x * Y + y];
    for (int n = 0; n < E->n; ++n) {
        double xd = (double)E->X[n], yd = (double)E->Y[n];
        double fx = xd - floor(xd), fy = yd - floor(yd);
        int sx = (int)ceil(c0 - xd), ix = (int)floor(os * fx);
        int sy = (int)ceil(c0 - yd), iy = (int)floor(os * fy);
        int sx2 = sx, ix2 = ix + 1, sy2 = sy, iy2 = iy + 1;
        if (ix == os - 1) { sx2 = sx - 1; ix2 = 0; }
        if (iy == os - 1) { sy2 = sy - 1; iy2 = 0; }
        float wy = (float)(1 - (fy - (double)iy / os) * os);
        float wx = (float)(1 - (fx - (double)ix / os) * os);
        for (int x = 0; x < X; ++x)
            for (int y = 0; y < Y; ++y) {
                float v1 = psf_get(r, (sy + y) + (sx + x) * s0 + iy * s01 + ix * s012, total);
                float v2 = psf_get(r, (sy + y) + (sx2 + x) * s0 + iy * s01 + ix2 * s012, total);
                float v3 = psf_get(r, (sy2 + y) + (sx + x) * s0 + iy2 * s01 + ix * s012, total);
                float v4 = psf_get(r, (sy2 + y) + (sx2 + x) * s0 + iy2 * s01 + ix2 * s012, total);
                float a = wx * v1 + (1.0f - wx) * v2;
                float b = wx * v3 + (1.0f - wx) * v4;
                M[y + x * Y] = M[y + x * Y] + E->I[n] * (wy * a + (1.0f - wy) * b);
            }
    }
}

static void state_model(orj *r, const oem *E, float *M)
{
    if (r->opt_model == 1) num_model(r, E, M);
    else model(r, E, M);
}

/* likelihood_ratio (:1650-1686).  r->M always equals the model of
 * E_Active.  The reference takes Params by value here, so until find_Birth
 * clears FirstCall it rebuilds M from E_Active on every call: the same
 * values, but the sampled-PSF model's index messages count each time. */
static float likelihood_ratio(orj *r)
{
    if (r->first_call && r->opt_model == 1) state_model(r, &r->A, r->M);
    state_model(r, &r->T, r->Mt);
    int N = r->X * r->Y;
    float tmp = 0;
    for (int n = 0; n < N; ++n) tmp += r->M[n] - r->Mt[n] + r->D[n] * O_LOG(r->Mt[n] / r->M[n]);
    return O_EXP(tmp);
}

/* Stat::genRand (:248-282). */
static float stat_rand(orj *r, const ostat *s)
{
    float R = urand(r);
    if (R <= 0) return 0;
    if (R >= 1) return s->ux[s->nu - 1];
    int si = -1;
    for (int i = 0; i < s->nu; ++i) {
        if (s->uc[i] - R > 0) {
            si = i;
            break;
        }
    }
    if (si == -1) {
        r->messages++;
        return 0;
    }
    if (si == 0) return 0;
    return (s->ux[si - 1] * (s->uc[si] - R) + s->ux[si] * (R - s->uc[si - 1])) /
           (s->uc[si] - s->uc[si - 1]);
}

static float sig_or_back(orj *r, int signal, float I)
{
    return signal == 1 ? stat_pdf(&r->sig, I, &r->messages) : stat_pdf(&r->back, I, &r->messages);
}

/* Distance test used by closest/closestMulti (:534,622): sqrt in double,
 * stored to float. */
static float em_dist_cl(const oem *e, int nn, int jj)
{
    float dx = e->X[nn] - e->X[jj], dy = e->Y[nn] - e->Y[jj];
    return (float)sqrt(O_POW2(dx) + O_POW2(dy));
}

/* Emitters::closest (:525-558). */
static int em_closest(orj *r, const oem *e, int jj, float dmin)
{
    int *ind = (int *)malloc((size_t)(e->n + 1) * sizeof(int));
    int num = 0, ii;
    for (int n = 0; n < e->n; ++n)
        if (n != jj && em_dist_cl(e, n, jj) < dmin) ind[num++] = n;
    if (num > 0) {
        float Ua = urand(r);
        int mm = (int)(Ua * num);
        if (mm > num - 1) mm = num - 1;
        ii = ind[mm];
    } else {
        int k = 0;
        for (int n = 0; n < e->n; ++n)
            if (n != jj) ind[k++] = n;
        float Ua = urand(r);
        int mm = (int)(Ua * (e->n - 1));
        if (mm > e->n - 2) mm = e->n - 2;
        ii = ind[mm];
    }
    free(ind);
    return ii;
}

/* Emitters::closestMulti (:615-650); returns the pick count. */
static int em_closest_multi(orj *r, const oem *e, int jj, float dmin, int *out)
{
    int *ind = (int *)malloc((size_t)(e->n + 1) * sizeof(int));
    int num = 0, np = 0;
    for (int n = 0; n < e->n; ++n)
        if (n != jj && em_dist_cl(e, n, jj) < dmin) ind[num++] = n;
    if (num > 0) {
        int Np;
        float Ua = urand(r);
        if (Ua < 1.0f / (float)num) {
            Np = num;
        } else {
            Np = (int)(Ua * num);
            if (Np > num - 1) Np = num - 1;
        }
        for (int n = 0; n < Np; ++n) {
            Ua = urand(r);
            int k = (int)(Ua * (num - n));
            if (k > num - n - 1) k = num - n - 1;
            out[np++] = ind[k];
            for (int q = k; q < num - n - 1; ++q) ind[q] = ind[q + 1];
        }
    }
    free(ind);
    return np;
}

/* Emitters::distance (:653-656): the squared sum is stored to float first. */
static float em_distance(const oem *e, int jj, int ii)
{
    float d = (float)(O_POW2(e->X[ii] - e->X[jj]) + O_POW2(e->Y[ii] - e->Y[jj]));
    return sqrtf(d);
}

/* RJMCMCChain::addEmitters (:290-322). */
static void chain_add(orj *r, int w, const oem *E, float LLR, float PR, int type, int acc)
{
    if (w == 0) {
        int ns = 0;
        for (int n = 0; n < E->n; ++n) ns += (E->S[n] == 1);
        ipush(&r->nsig_trace, E->n < 1 ? 0 : ns);
    }
    if (!r->record) return;
    ochain *c = &r->ch[w];
    fpush(&c->LLR, LLR);
    fpush(&c->PR, PR);
    ipush(&c->JumpType, type);
    ipush(&c->Accepted, acc);
    ipush(&c->N, E->n);
    fpush(&c->BG, E->BG);
    fpush(&c->ABG, E->ABG);
    fpush(&c->BBG, E->BBG);
    int state = c->Index.n == 0 ? 1 : c->Index.v[c->Index.n - 1] + 1;
    if (E->n < 1) {
        ipush(&c->Index, state);
        fpush(&c->Photons, 0);
        fpush(&c->X, -100);
        fpush(&c->Y, -100);
        ipush(&c->Signal, -1);
        return;
    }
    for (int n = 0; n < E->n; ++n) {
        ipush(&c->Index, state);
        fpush(&c->Photons, E->I[n]);
        fpush(&c->X, E->X[n] + r->p.DriftX);
        fpush(&c->Y, E->Y[n] + r->p.DriftY);
        ipush(&c->Signal, E->S[n]);
    }
}

/* RJMCMC::update_grids (:1629-1648). */
static void update_grids(orj *r)
{
    if (r->is_burnin || !r->pgrid) return;
    int Z = r->p.Grid_Zoom;
    for (int n = 0; n < r->A.n; ++n) {
        int x = kround((float)Z * (r->A.X[n] + r->p.DriftX));
        int y = kround((float)Z * (r->A.Y[n] + r->p.DriftY));
        float i = r->A.I[n];
        if (x >= 0 && x < r->X * Z && y >= 0 && y < r->Y * Z && i > r->p.Icutoff) {
            if (r->A.S[n] == 1)
                r->pgrid[x * r->Y * Z + y] = r->pgrid[x * r->Y * Z + y] + 1;
            else
                r->pback[x * r->Y * Z + y] = r->pback[x * r->Y * Z + y] + 1;
        }
    }
}

static void record2(orj *r, float LLR, float PR, int type, int acc)
{
    chain_add(r, 0, &r->A, LLR, PR, type, acc);
    chain_add(r, 1, &r->T, LLR, PR, type, acc);
}

static void accept_test(orj *r)
{
    em_copy(&r->A, &r->T);
    float *t = r->M;
    r->M = r->Mt;
    r->Mt = t;
}

static float nsignal(const oem *e)
{
    float NEm = 0;
    for (int n = 0; n < e->n; ++n) NEm = NEm + e->S[n];
    return NEm;
}

/* RJMCMC::jump (:752-970). */
static void mv_jump(orj *r)
{
    r->c.N_jump++;
    int type = 1, accept = 0;
    float LLR = 0, PR = 0, PrI = 1, PrBg, IPDF, IPDFtest;
    oem *A = &r->A, *T = &r->T;
    em_copy(T, A);
    if (A->n < 1) return;
    float Ua = urand(r);
    int nn = (int)(Ua * T->n);
    if (nn > T->n - 1) nn = T->n - 1;
    float Ub = urand(r);
    if ((double)Ub < 0.25) {
        type = 2;
        T->BG = T->BG + r->p.BG_std * randn(r);
        T->ABG = T->ABG + r->p.ABBG_std * randn(r);
        T->BBG = T->BBG + r->p.ABBG_std * randn(r);
    } else if ((double)Ub < 0.50 && (double)Ub >= 0.25) {
        if (A->n < 2) return;
        type = 10;
        int *cl = (int *)malloc((size_t)(A->n + 1) * sizeof(int));
        int Np = em_closest_multi(r, A, nn, 2 * r->p.PSFsigma, cl);
        if (Np == 0) {
            free(cl);
            return;
        }
        float I0 = A->I[nn];
        for (int i = 0; i < Np; ++i) I0 = I0 + A->I[cl[i]];
        float II0 = 0, XI0 = 0, YI0 = 0, XII0 = 0, YII0 = 0;
        for (int i = 0; i < Np; ++i) {
            int c = cl[i];
            if (A->S[c] == 1) {
                T->X[c] = A->X[c] + r->p.X_stdFg * randn(r);
                T->Y[c] = A->Y[c] + r->p.X_stdFg * randn(r);
                T->I[c] = (I0 / (float)(Np + 1)) * (0.15f * randn(r) + 1);
                IPDFtest = stat_pdf(&r->sig, T->I[c], &r->messages);
                IPDF = stat_pdf(&r->sig, A->I[c], &r->messages);
                PrI = PrI * IPDFtest / IPDF;
            } else {
                T->X[c] = A->X[c] + r->p.X_stdBg * randn(r);
                T->Y[c] = A->Y[c] + r->p.X_stdBg * randn(r);
                T->I[c] = (I0 / (float)(Np + 1)) * (0.15f * randn(r) + 1);
                IPDFtest = stat_pdf(&r->back, T->I[c], &r->messages);
                IPDF = stat_pdf(&r->back, A->I[c], &r->messages);
                PrI = PrI * IPDFtest / IPDF;
            }
            XI0 = XI0 + A->I[c] * A->X[c];
            YI0 = YI0 + A->I[c] * A->Y[c];
            XII0 = XII0 + T->I[c] * T->X[c];
            YII0 = YII0 + T->I[c] * T->Y[c];
            II0 = II0 + T->I[c];
        }
        T->I[nn] = I0 - II0;
        T->X[nn] = (XI0 + A->I[nn] * A->X[nn] - XII0) / T->I[nn];
        T->Y[nn] = (YI0 + A->I[nn] * A->Y[nn] - YII0) / T->I[nn];
        IPDFtest = sig_or_back(r, A->S[nn], T->I[nn]);
        IPDF = sig_or_back(r, A->S[nn], A->I[nn]);
        PrI = PrI * IPDFtest / IPDF;
        free(cl);
    } else if ((double)Ub >= 0.5 && (double)Ub < 0.75) {
        type = 3;
        int *ind = (int *)malloc((size_t)(A->n + 1) * sizeof(int));
        int NN = em_closest_multi(r, A, nn, 2 * r->p.PSFsigma, ind);
        ind[NN++] = nn;
        for (int i = 0; i < NN; ++i) {
            int c = ind[i];
            if (A->S[c] == 1) {
                r->c.N_jumpFg++;
                T->I[c] = T->I[c] + r->p.I_stdFg * randn(r);
                T->X[c] = T->X[c] + r->p.X_stdFg * randn(r);
                T->Y[c] = T->Y[c] + r->p.X_stdFg * randn(r);
                IPDFtest = stat_pdf(&r->sig, T->I[c], &r->messages);
                IPDF = stat_pdf(&r->sig, A->I[c], &r->messages);
                PrI = PrI * IPDFtest / IPDF;
            } else {
                r->c.N_jumpBg++;
                T->I[c] = T->I[c] + r->p.I_stdBg * randn(r);
                T->X[c] = T->X[c] + r->p.X_stdBg * randn(r);
                T->Y[c] = T->Y[c] + r->p.X_stdBg * randn(r);
                IPDFtest = stat_pdf(&r->back, T->I[c], &r->messages);
                IPDF = stat_pdf(&r->back, A->I[c], &r->messages);
                PrI = PrI * IPDFtest / IPDF;
            }
        }
        free(ind);
    } else {
        if (A->S[nn] == 1) {
            r->c.N_jumpFg++;
            T->I[nn] = T->I[nn] + r->p.I_stdFg * randn(r);
            T->X[nn] = T->X[nn] + r->p.X_stdFg * randn(r);
            T->Y[nn] = T->Y[nn] + r->p.X_stdFg * randn(r);
            IPDFtest = stat_pdf(&r->sig, T->I[nn], &r->messages);
            IPDF = stat_pdf(&r->sig, A->I[nn], &r->messages);
            PrI = IPDFtest / IPDF;
        } else {
            r->c.N_jumpBg++;
            T->I[nn] = T->I[nn] + r->p.I_stdBg * randn(r);
            T->X[nn] = T->X[nn] + r->p.X_stdBg * randn(r);
            T->Y[nn] = T->Y[nn] + r->p.X_stdBg * randn(r);
            IPDFtest = stat_pdf(&r->back, T->I[nn], &r->messages);
            IPDF = stat_pdf(&r->back, A->I[nn], &r->messages);
            PrI = IPDFtest / IPDF;
        }
    }
    if (!em_test(T, (int)r->p.Bnd_out, r->X, r->Y)) {
        record2(r, LLR, PR, type, accept);
        update_grids(r);
        return;
    }
    LLR = likelihood_ratio(r);
    float BgPDF = stat_pdf(&r->off, A->BG, &r->messages);
    float BgPDFtest = stat_pdf(&r->off, T->BG, &r->messages);
    PrBg = (BgPDFtest / BgPDF) * O_EXP(-(T->BBG * T->BBG - A->BBG * A->BBG) / 2) *
           O_EXP(-(T->ABG * T->ABG - A->ABG * A->ABG) / 2);
    PR = LLR * PrI * PrBg;
    accept = (urand(r) < PR);
    if (accept) {
        r->c.A_jump++;
        if (A->S[nn] == 1)
            r->c.A_jumpFg++;
        else
            r->c.A_jumpBg++;
        accept_test(r);
    }
    record2(r, LLR, PR, type, accept);
    update_grids(r);
}

/* RJMCMC::split (:972-1109). */
static void mv_split(orj *r)
{
    int type = 4, accept = 0;
    float LLR = 0, PR = 0;
    r->c.N_split++;
    oem *A = &r->A, *T = &r->T;
    em_copy(T, A);
    if (A->n < 1) return;
    float Ua = urand(r);
    int jj = (int)floorf((float)A->n * Ua);
    if (jj > A->n - 1) jj = A->n - 1;
    float Ijp = A->I[jj], mux = A->X[jj], muy = A->Y[jj];
    int BF = A->S[jj];
    if (BF == 1)
        r->c.N_splitFg++;
    else
        r->c.N_splitBg++;
    float u1 = urand(r);
    float u2 = r->p.Split_std * randn(r);
    float u3 = r->p.Split_std * randn(r);
    T->n = A->n;
    T->I[jj] = u1 * Ijp;
    T->X[jj] = mux + u2;
    T->Y[jj] = muy + u3;
    em_add(T, (1 - u1) * Ijp, mux - u1 * u2 / (1 - u1), muy - u1 * u3 / (1 - u1), BF);
    if (!em_test(T, (int)r->p.Bnd_out, r->X, r->Y)) {
        record2(r, LLR, PR, type, accept);
        update_grids(r);
        return;
    }
    LLR = likelihood_ratio(r);
    float tmp1 = 1, tmp2 = 1;
    tmp1 = tmp1 * sig_or_back(r, A->S[jj], A->I[jj]);
    tmp2 = tmp2 * sig_or_back(r, T->S[jj], T->I[jj]);
    tmp2 = tmp2 * sig_or_back(r, T->S[T->n - 1], T->I[T->n - 1]);
    float Norm1 = normpdf(u2, 0, r->p.Split_std);
    float Norm2 = normpdf(u3, 0, r->p.Split_std);
    float NEm = nsignal(A);
    float PrM = r->MeanN / (NEm + 1);
    float PrI = tmp2 / tmp1;
    float Area = (float)((r->X + r->p.Bnd_out) * (r->Y + r->p.Bnd_out));
    float PrX = 1 / Area;
    float Us = 1 / (Norm1 * Norm2);
    float Jacob = (float)((double)Ijp / O_POW2(1 - u1));
    PR = LLR * PrI * PrX * Us * Jacob * (r->P[1] / r->P[2]) * PrM;
    accept = (urand(r) < PR);
    if (accept) {
        r->c.A_split++;
        if (BF == 1)
            r->c.A_splitFg++;
        else
            r->c.A_splitBg++;
        accept_test(r);
    }
    record2(r, LLR, PR, type, accept);
    update_grids(r);
}

/* RJMCMC::merge (:1111-1255). */
static void mv_merge(orj *r)
{
    int type = 5, accept = 0;
    float LLR = 0, PR = 0;
    r->c.N_merge++;
    oem *A = &r->A, *T = &r->T;
    em_copy(T, A);
    if (A->n < 2) {
        update_grids(r);
        return;
    }
    float Ua = urand(r);
    int jj = (int)floorf((float)A->n * Ua);
    if (jj > A->n - 1) jj = A->n - 1;
    int ii = em_closest(r, A, jj, 3 * r->p.PSFsigma);
    if (A->S[jj] == 1)
        r->c.N_mergeFg++;
    else
        r->c.N_mergeBg++;
    if (em_distance(A, ii, jj) > 3 * r->p.PSFsigma) {
        update_grids(r);
        return;
    }
    float Ijp = A->I[jj] + A->I[ii];
    float muxjp = (A->I[jj] * A->X[jj] + A->I[ii] * A->X[ii]) / Ijp;
    float muyjp = (A->I[jj] * A->Y[jj] + A->I[ii] * A->Y[ii]) / Ijp;
    float u1 = A->I[jj] / Ijp;
    float u2 = A->X[jj] - muxjp;
    float u3 = A->Y[jj] - muyjp;
    T->I[jj] = Ijp;
    T->X[jj] = muxjp;
    T->Y[jj] = muyjp;
    float PDFfg = stat_pdf(&r->sig, Ijp, &r->messages);
    float PDFbg = stat_pdf(&r->back, Ijp, &r->messages);
    T->S[jj] = 1;
    if (PDFbg > PDFfg) T->S[jj] = 0;
    em_remove(T, ii);
    if (!em_test(T, (int)r->p.Bnd_out, r->X, r->Y)) {
        record2(r, LLR, PR, type, accept);
        update_grids(r);
        return;
    }
    LLR = likelihood_ratio(r);
    float tmp1 = 1, tmp2 = 1;
    tmp1 = tmp1 * sig_or_back(r, A->S[jj], A->I[jj]);
    tmp1 = tmp1 * sig_or_back(r, A->S[ii], A->I[ii]);
    if (ii > jj)
        tmp2 = tmp2 * sig_or_back(r, T->S[jj], T->I[jj]);
    else
        tmp2 = tmp2 * sig_or_back(r, T->S[jj - 1], T->I[jj - 1]);
    float Norm1 = normpdf(u2, 0, r->p.Split_std);
    float Norm2 = normpdf(u3, 0, r->p.Split_std);
    float NEm = nsignal(A);
    float PrI = tmp1 / tmp2;
    float Area = (float)((r->X + r->p.Bnd_out) * (r->Y + r->p.Bnd_out));
    float PrX = 1 / Area;
    float Us = 1 / (Norm1 * Norm2);
    float Jacob = (float)((double)Ijp / O_POW2(1 - u1));
    float PrM = r->MeanN / NEm;
    PR = LLR / (PrI * PrX * Jacob * Us * PrM * r->P[1] / r->P[2]);
    accept = (urand(r) < PR);
    if (accept) {
        if (A->S[jj] == 1)
            r->c.A_mergeFg++;
        else
            r->c.A_mergeBg++;
        r->c.A_merge++;
        accept_test(r);
    }
    record2(r, LLR, PR, type, accept);
    update_grids(r);
}

/* RJMCMC::find_Birth (:1688-1736); PixProb is always 1 (:1732). */
static void find_birth(orj *r, float *x, float *y)
{
    int N = r->X * r->Y;
    if (r->first_call && r->opt_model == 1) state_model(r, &r->A, r->M);
    r->first_call = 0;
    for (int n = 0; n < N; ++n) {
        float v = r->D[n] - r->M[n];
        r->resid[n] = (0.0f > v) ? 0.0f : v;
    }
    for (int n = 1; n < N; ++n) r->resid[n] += r->resid[n - 1];
    float rr = r->resid[N - 1] * urand(r);
    int ii;
    for (ii = 0; ii < N; ++ii)
        if (rr <= r->resid[ii]) break;
    *y = (float)(ii - r->Y * (ii / r->Y)) + urand(r) - 0.5f;
    *x = (float)(int)floorf((float)ii / (float)r->Y) + urand(r) - 0.5f;
}

/* RJMCMC::birth (:1258-1330). */
static void mv_birth(orj *r)
{
    int type = 6, accept = 0;
    float LLR = 0, PR = 0;
    r->c.N_birth++;
    oem *A = &r->A, *T = &r->T;
    em_copy(T, A);
    float x, y, PixProb = 1;
    int BF;
    find_birth(r, &x, &y);
    if (r->p.IsBackg == 1)
        BF = kround(urand(r));
    else
        BF = 1;
    float I_new;
    if (BF == 1) {
        r->c.N_birthFg++;
        I_new = stat_rand(r, &r->sig);
    } else {
        r->c.N_birthBg++;
        I_new = stat_rand(r, &r->back);
    }
    em_add(T, I_new, x, y, BF);
    if (!em_test(T, (int)r->p.Bnd_out, r->X, r->Y)) {
        record2(r, LLR, PR, type, accept);
        update_grids(r);
        return;
    }
    LLR = likelihood_ratio(r);
    float NEm = nsignal(A);
    float PrM = r->MeanN / (NEm + 1);
    PR = LLR * r->P[3] / (r->P[4] * (r->X + r->p.Bnd_out) * (r->Y + r->p.Bnd_out) * PixProb) * PrM;
    accept = (urand(r) < PR);
    if (accept) {
        if (BF == 1)
            r->c.A_birthFg++;
        else
            r->c.A_birthBg++;
        r->c.A_birth++;
        accept_test(r);
    }
    record2(r, LLR, PR, type, accept);
    update_grids(r);
}

/* RJMCMC::death (:1332-1387). */
static void mv_death(orj *r)
{
    int type = 7, accept = 0;
    float LLR = 0, PR = 0;
    r->c.N_death++;
    oem *A = &r->A, *T = &r->T;
    em_copy(T, A);
    if (A->n < 1) return;
    float Ua = urand(r);
    int jj = (int)floorf((float)A->n * Ua);
    if (jj > A->n - 1) jj = A->n - 1;
    if (A->S[jj] == 1)
        r->c.N_deathFg++;
    else
        r->c.N_deathBg++;
    em_remove(T, jj);
    LLR = likelihood_ratio(r);
    float NEm = nsignal(A);
    float PrM = NEm / r->MeanN;
    PR = LLR * (r->P[4] / r->P[3]) * PrM;
    accept = (urand(r) < PR);
    if (accept) {
        r->c.A_death++;
        if (A->S[jj] == 1)
            r->c.A_deathFg++;
        else
            r->c.A_deathBg++;
        accept_test(r);
    }
    record2(r, LLR, PR, type, accept);
    update_grids(r);
}

/* RJMCMC::gSplit (:1389-1485). */
static void mv_gsplit(orj *r)
{
    int type = 8, accept = 0;
    float LLR = 0, PR = 0, PrI = 1;
    oem *A = &r->A, *T = &r->T;
    if (A->n < 2) return;
    em_copy(T, A);
    float Ua = urand(r);
    int jj = (int)floorf((float)A->n * Ua);
    if (jj > A->n - 1) jj = A->n - 1;
    int *cl = (int *)malloc((size_t)(A->n + 2) * sizeof(int));
    int Np = em_closest_multi(r, A, jj, 2 * r->p.PSFsigma, cl);
    cl[Np++] = jj;
    if (Np == 1) {
        free(cl);
        return;
    }
    float I0 = 0, X0 = 0, Y0 = 0;
    for (int n = 0; n < Np; ++n) {
        I0 = I0 + A->I[cl[n]];
        X0 = X0 + A->X[cl[n]];
        Y0 = Y0 + A->Y[cl[n]];
    }
    float u1 = 0.3f * randn(r);
    float u2 = 0.3f * randn(r);
    float u3 = (1 / (float)Np) * urand(r);
    for (int n = 0; n < Np; ++n) {
        int c = cl[n];
        T->X[c] = (A->X[c] - u3 * (X0 / (float)Np + u1)) / (1 - u3);
        T->Y[c] = (A->Y[c] - u3 * (Y0 / (float)Np + u2)) / (1 - u3);
        T->I[c] = (1 - u3) * A->I[c];
    }
    em_add(T, u3 * I0, X0 / (float)Np + u1, Y0 / (float)Np + u2, 1);
    LLR = likelihood_ratio(r);
    float tmpCurrent, tmpProposed;
    for (int n = 0; n < Np; ++n) {
        int c = cl[n];
        tmpCurrent = sig_or_back(r, A->S[c], A->I[c]);
        tmpProposed = sig_or_back(r, T->S[n], T->I[c]);
        PrI = PrI * tmpProposed / tmpCurrent;
    }
    tmpProposed = sig_or_back(r, T->S[T->n - 1], T->I[T->n - 1]);
    PrI = PrI * (tmpProposed);
    float PDFu1 = normpdf(u1, 0.0f, 0.4f);
    float PDFu2 = normpdf(u2, 0.0f, 0.4f);
    float PDFu3 = (float)Np;
    float Us = 1 / (PDFu1 * PDFu2 * PDFu3);
    float NEm = nsignal(A);
    float PrM = r->MeanN / (NEm + 1);
    float Area = (float)((r->X + r->p.Bnd_out) * (r->Y + r->p.Bnd_out));
    float PrX = 1 / Area;
    float Jacob = I0 / O_POWF(1 - u3, (float)(Np + 1));
    PR = LLR * PrI * PrX * Us * Jacob * PrM * (r->P[5] / r->P[6]);
    accept = (urand(r) < PR);
    if (accept) accept_test(r);
    record2(r, LLR, PR, type, accept);
    update_grids(r);
    free(cl);
}

/* RJMCMC::gMerge (:1487-1584). */
static void mv_gmerge(orj *r)
{
    int type = 9, accept = 0;
    float LLR = 0, PR = 0, PrI = 1;
    oem *A = &r->A, *T = &r->T;
    if (A->n < 3) return;
    em_copy(T, A);
    float Ua = urand(r);
    int jj = (int)floorf((float)A->n * Ua);
    if (jj > A->n - 1) jj = A->n - 1;
    int *cl = (int *)malloc((size_t)(A->n + 1) * sizeof(int));
    int Np = em_closest_multi(r, A, jj, 3 * r->p.PSFsigma, cl);
    if (Np == 0) {
        free(cl);
        return;
    }
    float I0 = A->I[jj], X0 = A->X[jj], Y0 = A->Y[jj];
    for (int n = 0; n < Np; ++n) {
        I0 = I0 + A->I[cl[n]];
        X0 = X0 + A->X[cl[n]];
        Y0 = Y0 + A->Y[cl[n]];
    }
    (void)X0;
    (void)Y0;
    float U1, U2, U3, XX0 = 0, YY0 = 0;
    U3 = A->I[jj] / I0;
    for (int n = 0; n < Np; ++n) {
        int c = cl[n];
        T->I[c] = A->I[c] / (1 - U3);
        T->X[c] = U3 * A->X[jj] + (1 - U3) * A->X[c];
        XX0 = XX0 + U3 * A->X[jj] + (1 - U3) * A->X[c];
        T->Y[c] = U3 * A->Y[jj] + (1 - U3) * A->Y[c];
        YY0 = YY0 + U3 * A->Y[jj] + (1 - U3) * A->Y[c];
    }
    U1 = A->X[jj] - XX0 / Np;
    U2 = A->Y[jj] - YY0 / Np;
    float tmpProposed, tmpCurrent;
    for (int n = 0; n < Np; ++n) {
        int c = cl[n];
        tmpProposed = sig_or_back(r, T->S[c], T->I[c]);
        tmpCurrent = sig_or_back(r, A->S[c], A->I[c]);
        PrI = PrI * (tmpCurrent / tmpProposed);
    }
    tmpCurrent = sig_or_back(r, A->S[jj], A->I[jj]);
    PrI = PrI * tmpCurrent;
    em_remove(T, jj);
    LLR = likelihood_ratio(r);
    float PDFu1 = normpdf(U1, 0.0f, 0.4f);
    float PDFu2 = normpdf(U2, 0.0f, 0.4f);
    float PDFu3 = (float)Np;
    float Us = 1 / (PDFu1 * PDFu2 * PDFu3);
    float NEm = nsignal(A);
    float PrM = NEm / r->MeanN;
    float Area = (float)((r->X + r->p.Bnd_out) * (r->Y + r->p.Bnd_out));
    float PrX = 1 / Area;
    float Jacob = I0 / O_POWF(1 - U3, (float)(Np + 1));
    PR = LLR / (PrI * PrX * Us * Jacob * PrM * (r->P[5] / r->P[6]));
    if (PDFu1 == 0 || PDFu2 == 0) PR = -1;
    accept = (urand(r) < PR);
    if (accept) accept_test(r);
    record2(r, LLR, PR, type, accept);
    update_grids(r);
    free(cl);
}

/* RJMCMC::backFore (:1586-1627). */
static void mv_backfore(orj *r)
{
    oem *A = &r->A;
    if (A->n == 0) return;
    if (r->p.IsBackg == 0) return;
    float Ua = urand(r);
    int nn = (int)floorf((float)A->n * Ua);
    if (nn > A->n - 1) nn = A->n - 1;
    float BackP = stat_pdf(&r->back, A->I[nn], &r->messages);
    float SignalP = stat_pdf(&r->sig, A->I[nn], &r->messages);
    if (A->S[nn] == 1) {
        if (SignalP != 0) {
            float PrSig = BackP / SignalP;
            if (PrSig > urand(r)) A->S[nn] = 0;
        } else {
            A->S[nn] = 0;
        }
    } else {
        if (BackP != 0) {
            float PrSig = SignalP / BackP;
            if (PrSig > urand(r)) A->S[nn] = 1;
        } else {
            A->S[nn] = 1;
        }
    }
}

/* RJMCMC::start_Chain (:685-750). */
static void start_chain(orj *r)
{
    r->is_burnin = 1;
    for (int k = 0; k < 8; ++k) r->P[k] = r->p.P_Burnin[k];
    const float *V = r->PVB;
    for (int n = 0; n < r->p.N_Burnin; ++n) {
        float t = urand(r);
        if (t < V[0]) mv_jump(r);
        else if (t >= V[0] && t < V[1]) mv_split(r);
        else if (t >= V[1] && t < V[2]) mv_merge(r);
        else if (t >= V[2] && t < V[3]) mv_birth(r);
        else if (t >= V[3] && t < V[4]) mv_death(r);
        else if (t >= V[4] && t < V[5]) mv_gsplit(r);
        else if (t >= V[5] && t < V[6]) mv_gmerge(r);
        else mv_backfore(r);
    }
    r->is_burnin = 0;
    for (int k = 0; k < 8; ++k) r->P[k] = r->PVT[k];
    const float *W = r->PVT;
    for (int n = 0; n < r->p.N_Trials; ++n) {
        float t = urand(r);
        if (t < W[0]) mv_jump(r);
        else if (t >= W[0] && t < W[1]) mv_split(r);
        else if (t >= W[1] && t < W[2]) mv_merge(r);
        else if (t >= W[2] && t < W[3]) mv_birth(r);
        else if (t >= W[3] && t < W[4]) mv_death(r);
        else if (t >= V[4] && t < V[5]) mv_gsplit(r);
        else if (t >= V[5] && t < V[6]) mv_gmerge(r);
        else mv_backfore(r);
    }
}

/* Set-up of mexFunction (cRJMCMC.cpp:103-148) and make_Params (:14-50). */
static int orj_init(orj *r, const float *data, int xsize, int ysize, const bamf_emitters *e0,
                    const bamf_mcmc_params *p, const float *off, int loff, const float *sig,
                    int lsig, const float *back, int lback, const float *scmos,
                    const bamf_rng *rng, int record, int grids, const float *psf, int opt_model)
{
    memset(r, 0, sizeof *r);
    r->X = xsize;
    r->Y = ysize;
    r->D = data;
    r->p = *p;
    r->record = record;
    for (int ii = 0; ii < 8; ii++) {
        float PBtemp = 0, PTtemp = 0;
        for (int mm = 0; mm <= ii; mm++) {
            PBtemp = PBtemp + p->P_Burnin[mm];
            PTtemp = PTtemp + p->P_Trials[mm];
        }
        r->PVB[ii] = PBtemp;
        r->PVT[ii] = PTtemp;
    }
    r->MeanN = p->Rho * xsize * ysize;
    int N = xsize * ysize;
    float *z = NULL;
    if (!scmos) {
        z = (float *)calloc((size_t)N, sizeof(float));
        scmos = z;
    }
    r->scmos = scmos;
    em_reserve(&r->A, e0->N + 1);
    r->A.n = e0->N;
    for (int n = 0; n < e0->N; ++n) {
        r->A.I[n] = e0->I[n]; r->A.X[n] = e0->X[n]; r->A.Y[n] = e0->Y[n]; r->A.S[n] = 1;
    }
    r->A.BG = e0->BG;
    r->A.ABG = 0;
    r->A.BBG = 0;
    if (r->A.BG == 0) r->A.BG = 1;
    stat_init(&r->off, off, p->DX, loff);
    stat_init(&r->sig, sig, p->DX, lsig);
    stat_init(&r->back, back, p->DX, lback);
    r->M = (float *)malloc((size_t)N * sizeof(float));
    r->Mt = (float *)malloc((size_t)N * sizeof(float));
    r->resid = (float *)malloc((size_t)N * sizeof(float));
    if (grids) {
        size_t g = (size_t)N * p->Grid_Zoom * p->Grid_Zoom;
        r->pgrid = (float *)calloc(g, sizeof(float));
        r->pback = (float *)calloc(g, sizeof(float));
    }
    r->seed = rng->seed;
    r->chain = rng->chain_id;
    r->idx = rng->offset;
    bamf_counters *c = &r->c;
    c->N_jump = c->N_split = c->N_merge = c->N_birth = c->N_death = 1;
    c->N_jumpFg = c->N_splitFg = c->N_mergeFg = c->N_birthFg = c->N_deathFg = 1;
    c->N_jumpBg = c->N_splitBg = c->N_mergeBg = c->N_birthBg = c->N_deathBg = 1;
    /* M of the start state; the reference builds it at the first
     * likelihood_ratio / find_Birth call, which count its messages */
    r->first_call = 1;
    r->opt_model = opt_model;
    r->psf = psf;
    state_model(r, &r->A, r->M);
    r->messages = 0;
    return z != NULL; /* caller frees scmos if it was allocated here */
}

typedef struct {
    orj r;
    float *owned_scmos;
    uint32_t rng_offset;
} oresult;

static void orj_free(orj *r)
{
    stat_free(&r->off); stat_free(&r->sig); stat_free(&r->back);
    em_free(&r->A); em_free(&r->T);
    free(r->M); free(r->Mt); free(r->NX); free(r->NY); free(r->resid);
    chain_free(&r->ch[0]); chain_free(&r->ch[1]);
    free(r->nsig_trace.v);
    free(r->pgrid); free(r->pback);
}

static int args_ok(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                   const bamf_mcmc_params *p, const float *off, int loff, const float *sig,
                   int lsig, const float *back, int lback, const bamf_rng *rng)
{
    if (!data || !e0 || !p || !off || !sig || !back || !rng) return 0;
    if (xsize < 1 || ysize < 1 || loff < 1 || lsig < 1 || lback < 1) return 0;
    if (e0->N < 0 || (e0->N > 0 && (!e0->I || !e0->X || !e0->Y))) return 0;
    if (p->N_Burnin < 0 || p->N_Trials < 0 || p->Grid_Zoom < 0) return 0;
    return 1;
}

void *oracle_rjmcmc_run(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                        const bamf_mcmc_params *p, const float *off, int loff, const float *sig,
                        int lsig, const float *back, int lback, const float *scmos,
                        const bamf_rng *rng)
{
    return oracle_rjmcmc_run_model(data, xsize, ysize, e0, p, off, loff, sig, lsig, back, lback, scmos,
                                   NULL, 0, rng);
}

void *oracle_rjmcmc_run_model(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                              const bamf_mcmc_params *p, const float *off, int loff, const float *sig,
                              int lsig, const float *back, int lback, const float *scmos,
                              const float *sampled_psf, int opt_model, const bamf_rng *rng)
{
    if (!args_ok(data, xsize, ysize, e0, p, off, loff, sig, lsig, back, lback, rng)) return NULL;
    if (opt_model != 0 && opt_model != 1) return NULL;
    if (opt_model == 1) {
        long long total = 1;
        for (int k = 0; k < 4; ++k) {
            if (p->PSFsize[k] < 1) return NULL;
            total *= p->PSFsize[k];
        }
        if (!sampled_psf || total > 0x7fffffffLL) return NULL;
    }
    oresult *res = (oresult *)calloc(1, sizeof(oresult));
    int owned = orj_init(&res->r, data, xsize, ysize, e0, p, off, loff, sig, lsig, back, lback,
                         scmos, rng, 1, 1, sampled_psf, opt_model);
    if (owned) res->owned_scmos = (float *)res->r.scmos;
    res->rng_offset = rng->offset;
    start_chain(&res->r);
    return res;
}

int oracle_result_sizes(void *h, int64_t *sizes)
{
    oresult *o = (oresult *)h;
    if (!o || !sizes) return BAMF_ERR_INVALID_ARG;
    orj *r = &o->r;
    sizes[0] = r->ch[0].N.n;
    sizes[1] = r->ch[0].Index.n;
    sizes[2] = r->ch[1].N.n;
    sizes[3] = r->ch[1].Index.n;
    sizes[4] = (int64_t)r->X * r->Y * r->p.Grid_Zoom * r->p.Grid_Zoom;
    sizes[5] = (int64_t)(r->idx - o->rng_offset);
    sizes[6] = r->messages;
    return BAMF_OK;
}

int oracle_result_chain(void *h, int which, bamf_chain *out)
{
    oresult *o = (oresult *)h;
    if (!o || !out || which < 0 || which > 1) return BAMF_ERR_INVALID_ARG;
    ochain *c = &o->r.ch[which];
    if (c->N.n > out->capacity_entries || c->Index.n > out->capacity_records) return BAMF_ERR_CAPACITY;
    size_t ne = (size_t)c->N.n, nr = (size_t)c->Index.n;
    memcpy(out->N, c->N.v, ne * 4);
    memcpy(out->LLR, c->LLR.v, ne * 4);
    memcpy(out->PR, c->PR.v, ne * 4);
    memcpy(out->JumpType, c->JumpType.v, ne * 4);
    memcpy(out->Accepted, c->Accepted.v, ne * 4);
    memcpy(out->BG, c->BG.v, ne * 4);
    memcpy(out->ABG, c->ABG.v, ne * 4);
    memcpy(out->BBG, c->BBG.v, ne * 4);
    memcpy(out->Index, c->Index.v, nr * 4);
    memcpy(out->Photons, c->Photons.v, nr * 4);
    memcpy(out->X, c->X.v, nr * 4);
    memcpy(out->Y, c->Y.v, nr * 4);
    memcpy(out->Signal, c->Signal.v, nr * 4);
    out->n_entries = (int32_t)ne;
    out->n_records = (int32_t)nr;
    return BAMF_OK;
}

int oracle_result_grids(void *h, float *pgrid, float *pback)
{
    oresult *o = (oresult *)h;
    if (!o || !pgrid || !pback) return BAMF_ERR_INVALID_ARG;
    size_t g = (size_t)o->r.X * o->r.Y * o->r.p.Grid_Zoom * o->r.p.Grid_Zoom;
    memcpy(pgrid, o->r.pgrid, g * sizeof(float));
    memcpy(pback, o->r.pback, g * sizeof(float));
    return BAMF_OK;
}

int oracle_result_counters(void *h, bamf_counters *c)
{
    oresult *o = (oresult *)h;
    if (!o || !c) return BAMF_ERR_INVALID_ARG;
    *c = o->r.c;
    return BAMF_OK;
}

void oracle_result_free(void *h)
{
    oresult *o = (oresult *)h;
    if (!o) return;
    orj_free(&o->r);
    free(o->owned_scmos);
    free(o);
}

/* MAP emitter count of findMap.m:29-45 from the N-signal trace of the
 * accepted chain: the MEX output drops the last entry (cRJMCMC.cpp:174), so
 * Iter = entries - 1, and the mode (smallest on ties) is taken over
 * entries round(Iter/2) .. Iter (1-based). */
static int map_n_from_trace(const int32_t *t, int entries)
{
    int iter = entries - 1;
    if (iter < 1) return 0;
    int start = (iter + 1) / 2; /* MATLAB round(iter/2), iter >= 1 */
    if (start < 1) start = 1;
    int hist[BAMF_NMAX * 4 + 2];
    memset(hist, 0, sizeof hist);
    int maxn = 0;
    for (int k = start; k <= iter; ++k) {
        int v = t[k - 1];
        if (v > BAMF_NMAX * 4) v = BAMF_NMAX * 4;
        hist[v]++;
        if (v > maxn) maxn = v;
    }
    int best = 0;
    for (int v = 1; v <= maxn; ++v)
        if (hist[v] > hist[best]) best = v;
    return best;
}

typedef struct {
    const float *data;
    const int64_t *offsets;
    const int32_t *xs, *ys;
    const float *sigma;
    int n_rois;
    const bamf_mcmc_params *p;
    const float *off, *sig, *back;
    int loff, lsig, lback;
    float bg0;
    uint32_t seed;
    int next;
    pthread_mutex_t lock;
    int32_t *final_n, *map_n, *n_acc;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *j = (batch_job *)arg;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        int i = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (i >= j->n_rois) break;
        bamf_emitters e0 = {0, NULL, NULL, NULL, j->bg0};
        bamf_rng rng = {j->seed, (uint32_t)i, 0u};
        orj r;
        bamf_mcmc_params pi = *j->p;
        if (j->sigma) pi.PSFsigma = j->sigma[i];
        orj_init(&r, j->data + j->offsets[i], j->xs[i], j->ys[i], &e0, &pi, j->off, j->loff, j->sig,
                 j->lsig, j->back, j->lback, NULL, &rng, 0, 0, NULL, 0);
        float *owned = (float *)r.scmos;
        start_chain(&r);
        j->final_n[i] = r.A.n;
        j->map_n[i] = map_n_from_trace(r.nsig_trace.v, r.nsig_trace.n);
        bamf_counters *c = &r.c;
        j->n_acc[i] = c->A_jump + c->A_split + c->A_merge + c->A_birth + c->A_death;
        orj_free(&r);
        free(owned);
    }
    return NULL;
}

int oracle_rjmcmc_batch(const float *data, const int64_t *offsets, const int32_t *xs,
                        const int32_t *ys, const float *sigma, int n_rois, const bamf_mcmc_params *p,
                        const float *off, int loff, const float *sig, int lsig,
                        const float *back, int lback, float bg0, uint32_t seed, int threads,
                        int32_t *final_n, int32_t *map_n, int32_t *n_accepted)
{
    if (!data || !offsets || !xs || !ys || n_rois < 0 || !p || !final_n || !map_n || !n_accepted)
        return BAMF_ERR_INVALID_ARG;
    batch_job j = {data, offsets, xs, ys, sigma, n_rois, p, off, sig, back, loff, lsig, lback, bg0, seed, 0,
                   PTHREAD_MUTEX_INITIALIZER, final_n, map_n, n_accepted};
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, batch_worker, &j);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    return BAMF_OK;
}

/* The parity math on the host, for the device comparison (fn: 0 erf,
 * 1 log, 2 exp). */
int oracle_parity_math(int fn, const float *x, int n, float *out)
{
    if (!x || !out || n < 0 || fn < 0 || fn > 2) return BAMF_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i)
        out[i] = fn == 0 ? bamf_pm_erff(x[i]) : (fn == 1 ? bamf_pm_logf(x[i]) : bamf_pm_expf(x[i]));
    return BAMF_OK;
}
