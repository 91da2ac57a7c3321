/*
 * cRJMCMC_bamf.cpp - MEX gateway with the call signature of the reference's
 * cRJMCMC (source/c/cRJMCMC.cpp:52-308; called by @RJ/rjmcmc.m:102 and
 * @RJ/mcmc.m:142) that runs the chain on the GPU through the C ABI
 * (bamf_crjmcmc_host_model, include/bamf.h).
 *
 *   [PGrid, PBack, Chain, ProposedChain, Stat] = cRJMCMC_bamf(Data, E_active,
 *        MCMC, Xsize, Ysize, OffSetPDF, SignalPDF, BackPDF, sCMOScorr,
 *        SampledPSF, OptModel [, Arith [, Seed]])
 *
 * Inputs 1-11 are the reference's, with its types: Data, OffSetPDF,
 * SignalPDF, BackPDF, sCMOScorr and SampledPSF single; E_active a struct
 * with N, I, X, Y, BG; MCMC the struct rjmcmc.m:49-78 builds (P_Burnin and
 * P_Trials single[8], PSFsize int32 or uint32[4]).  Two optional inputs: Arith
 * 'exact' (default; the reference's chain bit for bit given the same
 * uniforms) or 'fast', and Seed (default 0; or [seed chain_id [offset]] to
 * name the uniform stream outright).
 *
 * Random numbers: the reference draws from glibc's rand(), which it never
 * seeds, so every MATLAB session replays the same sequence, continued from
 * call to call.  Here call k of a session (k = 0, 1, ...) takes the Philox
 * stream (Seed, chain id k) from its start: reproducible per session in the
 * same way, independent between calls.
 *
 * Outputs are marshalled as cRJMCMC.cpp:151-305 does: PGrid / PBack single
 * (Ysize*Zoom) x (Xsize*Zoom); Chain and ProposedChain L x 1 struct arrays
 * (L = recorded entries) whose first L-1 elements hold N, X, Y, Photons,
 * Signal, LLR, PR, JumpType, Accepted, BG, ABG, BBG as doubles (N = 0 for the
 * empty state, whose placeholder emitter is kept in X/Y/Photons/Signal; the
 * proposed chain takes LLR, PR, JumpType and Accepted from the accepted
 * chain) and whose last element is empty; Stat the 16 acceptance ratios.
 *
 * Unlike the reference, which reads whatever the pointers hold, every input
 * is checked: a wrong count, type or size, or a missing MCMC field, raises
 * a MATLAB error with identifier bamf:cRJMCMC:<what>, and so does an error
 * status of the library (bamf:cRJMCMC:status).
 */
#include <mex.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bamf.h"

namespace {

const char *const CHAIN_FIELDS[12] = {"N", "X", "Y", "Photons", "Signal", "LLR", "PR", "JumpType", "Accepted",
                                      "BG", "ABG", "BBG"};
const char *const STAT_FIELDS[16] = {"NTrials", "Accept_Jump", "Accept_Split", "Accept_Merge", "Accept_Birth",
                                     "Accept_Death", "Accept_JumpFg", "Accept_SplitFg", "Accept_MergeFg",
                                     "Accept_BirthFg", "Accept_DeathFg", "Accept_JumpBg", "Accept_SplitBg",
                                     "Accept_MergeBg", "Accept_BirthBg", "Accept_DeathBg"};

uint32_t g_calls = 0; /* calls of this session: the chain id of the next stream */

[[noreturn]] void fail(const char *what, const std::string &msg)
{
    const std::string id = std::string("bamf:cRJMCMC:") + what;
    mexErrMsgIdAndTxt(id.c_str(), "%s", msg.c_str());
    throw 0; /* not reached: mexErrMsgIdAndTxt does not return */
}

const float *single_data(const mxArray *a, const char *name, size_t min_elems)
{
    if (!a || !mxIsSingle(a)) fail("type", std::string(name) + " must be single");
    if (mxGetNumberOfElements(a) < min_elems)
        fail("size", std::string(name) + " has " + std::to_string(mxGetNumberOfElements(a)) +
                         " elements, needs " + std::to_string(min_elems));
    return (const float *)mxGetData(a);
}

/* the larger of rows and columns: how the reference takes a PDF's length
 * (cRJMCMC.cpp:77-98) */
int pdf_length(const mxArray *a)
{
    const mwSize m = mxGetM(a), n = mxGetN(a);
    return (int)(m > n ? m : n);
}

const mxArray *field(const mxArray *s, const char *name)
{
    const mxArray *f = mxGetField(s, 0, name);
    if (!f) fail("field", std::string("MCMC.") + name + " is missing");
    return f;
}

double scalar(const mxArray *s, const char *name)
{
    const mxArray *f = field(s, name);
    if (!mxIsNumeric(f) || mxGetNumberOfElements(f) < 1) fail("field", std::string("MCMC.") + name + " must be numeric");
    return mxGetScalar(f);
}

/* make_Params (cRJMCMC.cpp:14-50) */
void make_params(const mxArray *M, bamf_mcmc_params &p)
{
    if (!mxIsStruct(M)) fail("type", "MCMC must be a struct");
    std::memset(&p, 0, sizeof p);
    p.PSFsigma = (float)scalar(M, "PSFsigma");
    p.N_Trials = (int32_t)scalar(M, "N_Trials");
    p.N_Burnin = (int32_t)scalar(M, "N_Burnin");
    p.I_stdFg = (float)scalar(M, "I_stdFg");
    p.I_stdBg = (float)scalar(M, "I_stdBg");
    p.X_stdFg = (float)scalar(M, "X_stdFg");
    p.X_stdBg = (float)scalar(M, "X_stdBg");
    const float *pb = single_data(field(M, "P_Burnin"), "MCMC.P_Burnin", 8);
    const float *pt = single_data(field(M, "P_Trials"), "MCMC.P_Trials", 8);
    std::memcpy(p.P_Burnin, pb, sizeof p.P_Burnin);
    std::memcpy(p.P_Trials, pt, sizeof p.P_Trials);
    p.Rho = (float)scalar(M, "Rho");
    p.Bnd_out = (float)scalar(M, "Bnd_out");
    p.Grid_Zoom = (int32_t)scalar(M, "Grid_Zoom");
    p.Split_std = (float)scalar(M, "Split_std");
    p.Icutoff = (float)scalar(M, "Icutoff");
    p.BG_std = (float)scalar(M, "BG_std");
    p.ABBG_std = (float)scalar(M, "ABBG_std");
    p.DX = (float)scalar(M, "DX");
    p.DriftX = (float)scalar(M, "DriftX");
    p.DriftY = (float)scalar(M, "DriftY");
    const mxArray *ps = field(M, "PSFsize");
    if (!(mxGetClassID(ps) == mxINT32_CLASS || mxGetClassID(ps) == mxUINT32_CLASS) || mxGetNumberOfElements(ps) < 4)
        fail("field", "MCMC.PSFsize must be int32 or uint32 with 4 elements");
    std::memcpy(p.PSFsize, mxGetData(ps), sizeof p.PSFsize);
    p.IsBackg = (int32_t)scalar(M, "IsBackg");
}

/* E_active.I / X / Y as floats (single or double) */
std::vector<float> float_row(const mxArray *E, const char *name, int n)
{
    const mxArray *f = mxGetField(E, 0, name);
    if (!f) fail("field", std::string("E_active.") + name + " is missing");
    if ((mwSize)n > mxGetNumberOfElements(f)) fail("size", std::string("E_active.") + name + " is shorter than N");
    std::vector<float> v((size_t)n);
    if (mxIsSingle(f)) std::memcpy(v.data(), mxGetData(f), sizeof(float) * (size_t)n);
    else if (mxIsDouble(f))
        for (int k = 0; k < n; ++k) v[k] = (float)mxGetPr(f)[k];
    else fail("type", std::string("E_active.") + name + " must be single or double");
    return v;
}

mxArray *row(const float *v, int n)
{
    mxArray *a = mxCreateNumericMatrix(1, (mwSize)n, mxDOUBLE_CLASS, mxREAL);
    double *d = mxGetPr(a);
    for (int k = 0; k < n; ++k) d[k] = v[k];
    return a;
}

mxArray *row_i(const int32_t *v, int n)
{
    mxArray *a = mxCreateNumericMatrix(1, (mwSize)n, mxDOUBLE_CLASS, mxREAL);
    double *d = mxGetPr(a);
    for (int k = 0; k < n; ++k) d[k] = v[k];
    return a;
}

struct ChainBuf {
    std::vector<int32_t> N, JumpType, Accepted, Index, Signal;
    std::vector<float> LLR, PR, BG, ABG, BBG, Photons, X, Y;
    bamf_chain c;
    ChainBuf(int entries, int records)
    {
        N.resize(entries); JumpType.resize(entries); Accepted.resize(entries);
        LLR.resize(entries); PR.resize(entries); BG.resize(entries); ABG.resize(entries); BBG.resize(entries);
        Index.resize(records); Signal.resize(records); Photons.resize(records); X.resize(records); Y.resize(records);
        std::memset(&c, 0, sizeof c);
        c.capacity_entries = entries;
        c.capacity_records = records;
        c.N = N.data(); c.LLR = LLR.data(); c.PR = PR.data(); c.JumpType = JumpType.data();
        c.Accepted = Accepted.data(); c.BG = BG.data(); c.ABG = ABG.data(); c.BBG = BBG.data();
        c.Index = Index.data(); c.Photons = Photons.data(); c.X = X.data(); c.Y = Y.data(); c.Signal = Signal.data();
    }
};

/* cRJMCMC.cpp:159-276: an L x 1 struct array, entries 0..L-2 filled */
mxArray *marshal(const ChainBuf &b, const ChainBuf &acc)
{
    const int L = b.c.n_entries;
    mxArray *s = mxCreateStructMatrix((mwSize)L, 1, 12, (const char **)CHAIN_FIELDS);
    size_t rec = 0;
    for (int nn = 0; nn < L - 1; ++nn) {
        const int n = b.N[nn] < 1 ? 1 : b.N[nn]; /* the empty state keeps its placeholder record */
        const float *I = &b.Photons[rec];
        mxSetFieldByNumber(s, nn, 0, mxCreateDoubleScalar(I[0] == 0.0f ? 0.0 : (double)n));
        mxSetFieldByNumber(s, nn, 1, row(&b.X[rec], n));
        mxSetFieldByNumber(s, nn, 2, row(&b.Y[rec], n));
        mxSetFieldByNumber(s, nn, 3, row(I, n));
        mxSetFieldByNumber(s, nn, 4, row_i(&b.Signal[rec], n));
        mxSetFieldByNumber(s, nn, 5, mxCreateDoubleScalar((double)acc.LLR[nn]));
        mxSetFieldByNumber(s, nn, 6, mxCreateDoubleScalar((double)acc.PR[nn]));
        mxSetFieldByNumber(s, nn, 7, mxCreateDoubleScalar((double)acc.JumpType[nn]));
        mxSetFieldByNumber(s, nn, 8, mxCreateDoubleScalar((double)acc.Accepted[nn]));
        mxSetFieldByNumber(s, nn, 9, mxCreateDoubleScalar((double)b.BG[nn]));
        mxSetFieldByNumber(s, nn, 10, mxCreateDoubleScalar((double)b.ABG[nn]));
        mxSetFieldByNumber(s, nn, 11, mxCreateDoubleScalar((double)b.BBG[nn]));
        rec += (size_t)n;
    }
    return s;
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs < 11 || nrhs > 13) fail("nrhs", "cRJMCMC_bamf takes 11 inputs (the reference's) plus optional Arith, Seed");
    if (nlhs > 5) fail("nlhs", "cRJMCMC_bamf has 5 outputs");
    bamf_mcmc_params p;
    make_params(prhs[2], p);
    const int Xsize = (int)mxGetScalar(prhs[3]);
    const int Ysize = (int)mxGetScalar(prhs[4]);
    if (Xsize < 1 || Ysize < 1) fail("size", "Xsize and Ysize must be positive");
    const size_t npix = (size_t)Xsize * (size_t)Ysize;
    const float *data = single_data(prhs[0], "Data", npix);
    const float *off = single_data(prhs[5], "OffSetPDF", 1);
    const float *sig = single_data(prhs[6], "SignalPDF", 1);
    const float *back = single_data(prhs[7], "BackPDF", 1);
    const float *scmos = single_data(prhs[8], "sCMOScorr", npix);
    const int opt_model = (int)mxGetScalar(prhs[10]);
    const float *psf = nullptr;
    if (opt_model == 1) {
        size_t need = 1;
        for (int k = 0; k < 4; ++k) need *= (size_t)(p.PSFsize[k] > 0 ? p.PSFsize[k] : 0);
        psf = single_data(prhs[9], "SampledPSF", need);
    } else if (opt_model != 0) {
        fail("OptModel", "OptModel must be 0 (Gaussian PSF) or 1 (sampled PSF)");
    }
    int arith = BAMF_ARITH_EXACT;
    if (nrhs >= 12) {
        char buf[16] = {0};
        if (!mxIsChar(prhs[11]) || mxGetString(prhs[11], buf, sizeof buf)) fail("Arith", "Arith must be 'exact' or 'fast'");
        if (!std::strcmp(buf, "fast")) arith = BAMF_ARITH_FAST;
        else if (std::strcmp(buf, "exact")) fail("Arith", "Arith must be 'exact' or 'fast'");
    }
    /* Seed: a scalar (the session's next chain id), or [seed chain_id] /
     * [seed chain_id offset] naming the stream outright */
    uint32_t seed = 0, chain = 0, offset = 0;
    bool named = false;
    if (nrhs >= 13) {
        const mxArray *S = prhs[12];
        const mwSize ns = mxGetNumberOfElements(S);
        if (!mxIsDouble(S) || ns < 1 || ns > 3) fail("Seed", "Seed must be a double scalar or [seed chain_id [offset]]");
        const double *v = mxGetPr(S);
        for (mwSize k = 0; k < ns; ++k)
            if (!(v[k] >= 0 && v[k] <= 4294967295.0 && v[k] == std::floor(v[k])))
                fail("Seed", "Seed values must be integers in [0, 2^32)");
        seed = (uint32_t)v[0];
        if (ns >= 2) { chain = (uint32_t)v[1]; named = true; }
        if (ns == 3) offset = (uint32_t)v[2];
    }

    const mxArray *E = prhs[1];
    if (!mxIsStruct(E)) fail("type", "E_active must be a struct");
    const mxArray *fN = mxGetField(E, 0, "N"), *fBG = mxGetField(E, 0, "BG");
    if (!fN || !fBG) fail("field", "E_active needs N, I, X, Y and BG");
    const int n0 = (int)mxGetScalar(fN);
    if (n0 < 0) fail("size", "E_active.N must not be negative");
    std::vector<float> I = float_row(E, "I", n0), X = float_row(E, "X", n0), Y = float_row(E, "Y", n0);
    bamf_emitters e0 = {n0, I.data(), X.data(), Y.data(), (float)mxGetScalar(fBG)};
    const bamf_rng rng = {seed, named ? chain : g_calls++, offset};

    const int steps = p.N_Burnin + p.N_Trials;
    const int entries = steps + 1;
    ChainBuf acc(entries, entries * BAMF_NMAX), prop(entries, entries * BAMF_NMAX);
    const size_t gsz = npix * (size_t)p.Grid_Zoom * (size_t)p.Grid_Zoom;
    const mwSize gd[2] = {(mwSize)Ysize * (mwSize)p.Grid_Zoom, (mwSize)Xsize * (mwSize)p.Grid_Zoom};
    mxArray *pg = mxCreateNumericArray(2, gd, mxSINGLE_CLASS, mxREAL);
    mxArray *pbk = mxCreateNumericArray(2, gd, mxSINGLE_CLASS, mxREAL);
    bamf_counters cnt;
    const bamf_status st = bamf_crjmcmc_host_model(
        data, Xsize, Ysize, &e0, &p, off, pdf_length(prhs[5]), sig, pdf_length(prhs[6]), back, pdf_length(prhs[7]),
        scmos, psf, opt_model, &rng, arith, gsz ? (float *)mxGetData(pg) : nullptr,
        gsz ? (float *)mxGetData(pbk) : nullptr, &acc.c, &prop.c, &cnt);
    if (st != BAMF_OK) {
        mxDestroyArray(pg);
        mxDestroyArray(pbk);
        fail("status", std::string("bamf_crjmcmc_host_model returned ") + std::to_string(st) + " " + bamf_last_error());
    }
    plhs[0] = pg;
    if (nlhs > 1) plhs[1] = pbk; else mxDestroyArray(pbk);
    if (nlhs > 2) plhs[2] = marshal(acc, acc);
    if (nlhs > 3) plhs[3] = marshal(prop, acc);
    if (nlhs > 4) {
        mxArray *s = mxCreateStructMatrix(1, 1, 16, (const char **)STAT_FIELDS);
        const int32_t *c = &cnt.N_jump; /* bamf_counters order: N_*, A_*, then Fg, Bg */
        mxSetFieldByNumber(s, 0, 0, mxCreateDoubleScalar((double)p.N_Trials + p.N_Burnin));
        for (int g = 0; g < 3; ++g)
            for (int m = 0; m < 5; ++m)
                mxSetFieldByNumber(s, 0, 1 + 5 * g + m, mxCreateDoubleScalar((double)c[10 * g + 5 + m] / c[10 * g + m]));
        plhs[4] = s;
    }
}
