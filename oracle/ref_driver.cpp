/*
 * ref_driver.cpp - TEST INFRASTRUCTURE.  Runs the unmodified reference
 * sampler (source/c/LibRJMCMC.cpp, compiled from the reference tree by
 * oracle/Makefile into oracle/_ref/) on one ROI and hands its raw outputs to
 * the tests through a small C API.  Nothing in the product links this.
 *
 * The set-up mirrors the MEX gateway mexFunction (source/c/cRJMCMC.cpp):
 *   - make_Params (:14-50): scalar fields, cumulative PV_Burnin/PV_Trials,
 *     PSFsizeV;
 *   - MeanN = Rho * Xsize * Ysize (:116);
 *   - Emitters(N, I, X, Y, BG, 0, 0) with BG == 0 replaced by 1 (:124-133);
 *   - the three Stat tables from the PDFs (:135-137);
 *   - RJMCMC(...), IsBurnin = 0, state and tables assigned, start_Chain()
 *     (:139-148).
 * Outputs are the raw RJMCMCChain vectors of Chain and Chain_Test, PGridV,
 * PBackV and the 30 counters, before the MEX marshalling (:151-305), which
 * the project restates separately.
 *
 * The uniform stream: the shim header renames rand() to bamf_ref_rand(),
 * defined here from the Philox stream (include/bamf_philox.h).  State is
 * thread-local so that tests may run several ROIs on host threads.
 */
/* standard headers the batch runner needs, before the reference header
 * defines its min/max/pi macros */
#include <atomic>
#include <thread>

#include "LibRJMCMCreturn.hpp"

#include <cstdarg>
#include <cstdint>
#include <cstring>

#include "bamf.h"
#include "bamf_philox.h"

static thread_local uint32_t g_seed = 0, g_chain = 0, g_index = 0;
static thread_local int g_messages = 0;

extern "C" int bamf_ref_rand(void)
{
    return (int)bamf_stream_u31(g_seed, g_chain, g_index++);
}

extern "C" int bamf_ref_mex_printf(const char *fmt, ...)
{
    (void)fmt;
    ++g_messages;
    return 0;
}

namespace {

struct RefResult {
    std::vector<float> LLR[2], PR[2], BG[2], ABG[2], BBG[2], Photons[2], X[2], Y[2];
    std::vector<int> N[2], JumpType[2], Accepted[2], Index[2], Signal[2];
    std::vector<float> pgrid, pback;
    bamf_counters counters;
    int messages = 0;
    uint32_t rand_used = 0;
};

void take_chain(RefResult &r, int w, const RJMCMCChain &c)
{
    r.LLR[w] = c.LLR; r.PR[w] = c.PR; r.BG[w] = c.BG; r.ABG[w] = c.ABG; r.BBG[w] = c.BBG;
    r.Photons[w] = c.Photons; r.X[w] = c.X; r.Y[w] = c.Y;
    r.N[w] = c.N; r.JumpType[w] = c.JumpType; r.Accepted[w] = c.Accepted;
    r.Index[w] = c.Index; r.Signal[w] = c.Signal;
}

}  // namespace

extern "C" void *ref_rjmcmc_run_model(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                                      const bamf_mcmc_params *p, const float *off, int loff,
                                      const float *sig, int lsig, const float *back, int lback,
                                      const float *scmos, const float *sampled_psf, int opt_model,
                                      const bamf_rng *rng);

extern "C" void *ref_rjmcmc_run(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                                const bamf_mcmc_params *p, const float *off, int loff,
                                const float *sig, int lsig, const float *back, int lback,
                                const float *scmos, const bamf_rng *rng)
{
    return ref_rjmcmc_run_model(data, xsize, ysize, e0, p, off, loff, sig, lsig, back, lback, scmos, nullptr,
                                0, rng);
}

/* cRJMCMC's SampledPSF (prhs[9]) and OptModel (prhs[10]) inputs
 * (cRJMCMC.cpp:73-74); a null sampled_psf passes zeros, as rjmcmc.m:82-84
 * does for the Gaussian model. */
extern "C" void *ref_rjmcmc_run_model(const float *data, int xsize, int ysize, const bamf_emitters *e0,
                                      const bamf_mcmc_params *p, const float *off, int loff,
                                      const float *sig, int lsig, const float *back, int lback,
                                      const float *scmos, const float *sampled_psf, int opt_model,
                                      const bamf_rng *rng)
{
    if (!data || !e0 || !p || !off || !sig || !back || !rng || xsize < 1 || ysize < 1 || loff < 1 ||
        lsig < 1 || lback < 1)
        return nullptr;
    if ((opt_model != 0 && opt_model != 1) || (opt_model == 1 && !sampled_psf)) return nullptr;
    for (int k = 0; k < 4; ++k)
        if (p->PSFsize[k] < 1) return nullptr;
    g_seed = rng->seed;
    g_chain = rng->chain_id;
    g_index = rng->offset;
    g_messages = 0;

    MCMC_Parameters Params;
    float pb[8], pt[8];
    std::memcpy(pb, p->P_Burnin, sizeof pb);
    std::memcpy(pt, p->P_Trials, sizeof pt);
    int psfsize[4];
    std::memcpy(psfsize, p->PSFsize, sizeof psfsize);
    Params.PSFsigma = p->PSFsigma;
    Params.N_Trials = p->N_Trials;
    Params.N_Burnin = p->N_Burnin;
    Params.I_stdFg = p->I_stdFg;
    Params.I_stdBg = p->I_stdBg;
    Params.X_stdFg = p->X_stdFg;
    Params.X_stdBg = p->X_stdBg;
    Params.P_Burnin = pb;
    Params.P_Trials = pt;
    Params.Rho = p->Rho;
    Params.Bnd_out = p->Bnd_out;
    Params.Grid_Zoom = p->Grid_Zoom;
    Params.Split_std = p->Split_std;
    Params.Icutoff = p->Icutoff;
    Params.BG_std = p->BG_std;
    Params.ABBG_std = p->ABBG_std;
    Params.DX = p->DX;
    Params.DriftX = p->DriftX;
    Params.DriftY = p->DriftY;
    Params.PSFsize = psfsize;
    Params.IsBackg = p->IsBackg;
    for (int ii = 0; ii < 8; ii++) {
        float PBtemp = 0, PTtemp = 0;
        for (int mm = 0; mm <= ii; mm++) {
            PBtemp = PBtemp + Params.P_Burnin[mm];
            PTtemp = PTtemp + Params.P_Trials[mm];
        }
        Params.PV_Burnin.push_back(PBtemp);
        Params.PV_Trials.push_back(PTtemp);
    }
    for (int ii = 0; ii < 4; ii++) Params.PSFsizeV.push_back(Params.PSFsize[ii]);

    float MeanN = Params.Rho * xsize * ysize;
    Emitters E_Active = Emitters(e0->N, const_cast<float *>(e0->I), const_cast<float *>(e0->X),
                                 const_cast<float *>(e0->Y), e0->BG, 0, 0);
    if (E_Active.BG == 0) E_Active.BG = 1;
    Stat OffgStat = Stat(const_cast<float *>(off), Params.DX, loff);
    Stat SignalStat = Stat(const_cast<float *>(sig), Params.DX, lsig);
    Stat BackStat = Stat(const_cast<float *>(back), Params.DX, lback);

    std::vector<float> zeros_scmos;
    if (!scmos) {
        zeros_scmos.assign((size_t)xsize * ysize, 0.0f);
        scmos = zeros_scmos.data();
    }
    size_t psfn = (size_t)psfsize[0] * psfsize[1] * psfsize[2] * psfsize[3];
    std::vector<float> psf_buf(psfn, 0.0f);
    if (sampled_psf) psf_buf.assign(sampled_psf, sampled_psf + psfn);

    RefResult *res = new RefResult();
    {
        RJMCMC RJ = RJMCMC(const_cast<float *>(data), Params, xsize, ysize, const_cast<float *>(scmos),
                           MeanN, psf_buf.data(), opt_model);
        RJ.IsBurnin = 0;
        RJ.E_Active = E_Active;
        RJ.OffgStat = OffgStat;
        RJ.BackStat = BackStat;
        RJ.SignalStat = SignalStat;
        RJ.start_Chain();
        take_chain(*res, 0, RJ.Chain);
        take_chain(*res, 1, RJ.Chain_Test);
        res->pgrid = RJ.PGridV;
        res->pback = RJ.PBackV;
        bamf_counters &c = res->counters;
        c.N_jump = RJ.N_jump; c.N_split = RJ.N_split; c.N_merge = RJ.N_merge;
        c.N_birth = RJ.N_birth; c.N_death = RJ.N_death;
        c.A_jump = RJ.A_jump; c.A_split = RJ.A_split; c.A_merge = RJ.A_merge;
        c.A_birth = RJ.A_birth; c.A_death = RJ.A_death;
        c.N_jumpFg = RJ.N_jumpFg; c.N_splitFg = RJ.N_splitFg; c.N_mergeFg = RJ.N_mergeFg;
        c.N_birthFg = RJ.N_birthFg; c.N_deathFg = RJ.N_deathFg;
        c.A_jumpFg = RJ.A_jumpFg; c.A_splitFg = RJ.A_splitFg; c.A_mergeFg = RJ.A_mergeFg;
        c.A_birthFg = RJ.A_birthFg; c.A_deathFg = RJ.A_deathFg;
        c.N_jumpBg = RJ.N_jumpBg; c.N_splitBg = RJ.N_splitBg; c.N_mergeBg = RJ.N_mergeBg;
        c.N_birthBg = RJ.N_birthBg; c.N_deathBg = RJ.N_deathBg;
        c.A_jumpBg = RJ.A_jumpBg; c.A_splitBg = RJ.A_splitBg; c.A_mergeBg = RJ.A_mergeBg;
        c.A_birthBg = RJ.A_birthBg; c.A_deathBg = RJ.A_deathBg;
    }
    res->messages = g_messages;
    res->rand_used = g_index - rng->offset;
    return res;
}

/* sizes: [entries, records, entries_test, records_test, grid_elems,
 *         uniforms_used, messages] */
extern "C" int ref_result_sizes(void *h, int64_t *sizes)
{
    RefResult *r = static_cast<RefResult *>(h);
    if (!r) return BAMF_ERR_INVALID_ARG;
    sizes[0] = (int64_t)r->N[0].size();
    sizes[1] = (int64_t)r->Index[0].size();
    sizes[2] = (int64_t)r->N[1].size();
    sizes[3] = (int64_t)r->Index[1].size();
    sizes[4] = (int64_t)r->pgrid.size();
    sizes[5] = (int64_t)r->rand_used;
    sizes[6] = (int64_t)r->messages;
    return BAMF_OK;
}

extern "C" int ref_result_chain(void *h, int which, bamf_chain *out)
{
    RefResult *r = static_cast<RefResult *>(h);
    if (!r || !out || which < 0 || which > 1) return BAMF_ERR_INVALID_ARG;
    int ne = (int)r->N[which].size(), nr = (int)r->Index[which].size();
    if (ne > out->capacity_entries || nr > out->capacity_records) return BAMF_ERR_CAPACITY;
    for (int i = 0; i < ne; ++i) {
        out->N[i] = r->N[which][i];
        out->LLR[i] = r->LLR[which][i];
        out->PR[i] = r->PR[which][i];
        out->JumpType[i] = r->JumpType[which][i];
        out->Accepted[i] = r->Accepted[which][i];
        out->BG[i] = r->BG[which][i];
        out->ABG[i] = r->ABG[which][i];
        out->BBG[i] = r->BBG[which][i];
    }
    for (int i = 0; i < nr; ++i) {
        out->Index[i] = r->Index[which][i];
        out->Photons[i] = r->Photons[which][i];
        out->X[i] = r->X[which][i];
        out->Y[i] = r->Y[which][i];
        out->Signal[i] = r->Signal[which][i];
    }
    out->n_entries = ne;
    out->n_records = nr;
    return BAMF_OK;
}

extern "C" int ref_result_grids(void *h, float *pgrid, float *pback)
{
    RefResult *r = static_cast<RefResult *>(h);
    if (!r || !pgrid || !pback) return BAMF_ERR_INVALID_ARG;
    std::memcpy(pgrid, r->pgrid.data(), r->pgrid.size() * sizeof(float));
    std::memcpy(pback, r->pback.data(), r->pback.size() * sizeof(float));
    return BAMF_OK;
}

extern "C" int ref_result_counters(void *h, bamf_counters *c)
{
    RefResult *r = static_cast<RefResult *>(h);
    if (!r || !c) return BAMF_ERR_INVALID_ARG;
    *c = r->counters;
    return BAMF_OK;
}

extern "C" void ref_result_free(void *h) { delete static_cast<RefResult *>(h); }

/* A batch of ROIs through the reference sampler on host threads, the way the
 * @RJ pipeline runs them (one cRJMCMC call per ROI, RJ.m:217-244 parfor over
 * workers): ROI k with the empty start of rjmcmc.m:43-47 (BG = bg0), its own
 * PSF sigma, uniform stream (seed, k, 0).  Per ROI: final emitter count, MAP
 * count (mode of the Signal==1 count over entries round(L/2)..L of the
 * accepted chain without its last entry, findMap.m:29-45) and accepted
 * moves.  Same interface as the port's oracle_rjmcmc_batch. */
static int ref_map_n(const RefResult &r)
{
    const std::vector<int> &N = r.N[0];
    const int entries = (int)N.size();
    const int iter = entries - 1;
    if (iter < 1) return 0;
    const int start = (iter + 1) / 2 < 1 ? 1 : (iter + 1) / 2;
    std::vector<int> nsig(entries, 0);
    size_t rec = 0;
    for (int e = 0; e < entries; ++e) {
        const int n = N[e] < 1 ? 1 : N[e];
        int s = 0;
        for (int k = 0; k < n && rec + k < r.Signal[0].size(); ++k) s += r.Signal[0][rec + k] == 1;
        nsig[e] = N[e] < 1 ? 0 : s;
        rec += (size_t)n;
    }
    std::vector<int> hist(BAMF_NMAX * 4 + 2, 0);
    int maxn = 0;
    for (int k = start; k <= iter; ++k) {
        int v = nsig[k - 1];
        if (v > BAMF_NMAX * 4) v = BAMF_NMAX * 4;
        hist[v]++;
        if (v > maxn) maxn = v;
    }
    int best = 0;
    for (int v = 1; v <= maxn; ++v)
        if (hist[v] > hist[best]) best = v;
    return best;
}

extern "C" int ref_rjmcmc_batch(const float *data, const int64_t *offsets, const int32_t *xs, const int32_t *ys,
                                const float *sigma, int n_rois, const bamf_mcmc_params *p, const float *off,
                                int loff, const float *sig, int lsig, const float *back, int lback, float bg0,
                                uint32_t seed, int threads, int32_t *final_n, int32_t *map_n, int32_t *n_accepted)
{
    if (!data || !offsets || !xs || !ys || n_rois < 0 || !p || !final_n || !map_n || !n_accepted)
        return BAMF_ERR_INVALID_ARG;
    std::atomic<int> next(0);
    auto worker = [&]() {
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n_rois) break;
            bamf_emitters e0 = {0, nullptr, nullptr, nullptr, bg0};
            bamf_rng rng = {seed, (uint32_t)i, 0u};
            bamf_mcmc_params pk = *p;
            if (sigma) pk.PSFsigma = sigma[i];
            RefResult *r = static_cast<RefResult *>(ref_rjmcmc_run_model(
                data + offsets[i], xs[i], ys[i], &e0, &pk, off, loff, sig, lsig, back, lback, nullptr, nullptr, 0,
                &rng));
            if (!r) {
                final_n[i] = map_n[i] = n_accepted[i] = -1;
                continue;
            }
            final_n[i] = r->N[0].empty() ? 0 : r->N[0].back();
            map_n[i] = ref_map_n(*r);
            const bamf_counters &c = r->counters;
            n_accepted[i] = c.A_jump + c.A_split + c.A_merge + c.A_birth + c.A_death;
            delete r;
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(worker);
    for (auto &t : th) t.join();
    return BAMF_OK;
}
