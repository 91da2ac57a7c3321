/*
 * bamf_driver.cpp - standalone C++ driver of libbamf_gb300.so through its C
 * ABI (include/bamf.h), no MATLAB and no Python:
 *
 *   bamf_driver rjmcmc <input> <output>
 *       one cRJMCMC call (bamf_crjmcmc_host: the MEX function cRJMCMC of
 *       source/c/cRJMCMC.cpp:52-308 without MATLAB) on the ROI, settings,
 *       start state, priors and uniform stream in <input>; writes the raw
 *       chains (accepted and proposed), the posterior grids and the 30
 *       counters to <output> (file layouts below)
 *   bamf_driver batch <n_rois> <jumps> [seed]
 *       generates n_rois ROIs like the batched uneven workload (sides
 *       {8,12,16,20,24}, N ~ Poisson(U[0,12]), sigma U[1.1,1.5], I ~
 *       LogN(ln 1000, 0.4), background U[5,50], Poisson noise), runs them
 *       through bamf_rjmcmc_batch_host with `jumps` burn-in and trial jumps
 *       (fast arithmetic, the reference's moves) and prints one JSON line:
 *       ROIs/s through the host entry point, mean MAP and true counts
 *
 * <input> (little-endian): "BAMFRJ1\0"; int32 xsize, ysize; the
 * bamf_mcmc_params struct as laid out by this ABI; int32 N; float BG;
 * float I[N], X[N], Y[N]; uint32 seed, chain_id, offset; int32 arith;
 * int32 L then float[L] for each of OffSetPDF, SignalPDF, BackPDF;
 * float data[ysize*xsize] (y fastest).
 * <output>: "BAMFRO1\0"; int32 status; for Chain then Chain_Test: int32
 * n_entries, n_records, then N, LLR, PR, JumpType, Accepted, BG, ABG, BBG
 * (n_entries each) and Index, Photons, X, Y, Signal (n_records each);
 * int64 grid size G, float PGrid[G], PBack[G]; int32 counters[30].
 */
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "bamf.h"

namespace {

struct Reader {
    FILE *f;
    template <typename T>
    bool get(T *v, size_t n = 1) { return n == 0 || std::fread(v, sizeof(T), n, f) == n; }
};

template <typename T>
void put(FILE *f, const T *v, size_t n) { if (n) std::fwrite(v, sizeof(T), n, f); }

int usage()
{
    std::fprintf(stderr, "usage: bamf_driver rjmcmc <input> <output>\n"
                         "       bamf_driver batch <n_rois> <jumps> [seed]\n");
    return 2;
}

int run_rjmcmc(const char *in_path, const char *out_path)
{
    FILE *f = std::fopen(in_path, "rb");
    if (!f) { std::perror(in_path); return 1; }
    Reader r{f};
    char magic[8];
    int32_t xs = 0, ys = 0, n0 = 0, arith = 0;
    float bg = 0;
    bamf_mcmc_params p;
    bamf_rng rng;
    bool ok = r.get(magic, 8) && !std::memcmp(magic, "BAMFRJ1", 8) && r.get(&xs) && r.get(&ys) && r.get(&p) &&
              r.get(&n0) && r.get(&bg) && n0 >= 0 && n0 <= BAMF_NMAX && xs > 0 && ys > 0 && xs <= 4096 && ys <= 4096;
    std::vector<float> I(ok ? n0 : 0), X(ok ? n0 : 0), Y(ok ? n0 : 0), pdf[3], data;
    ok = ok && r.get(I.data(), n0) && r.get(X.data(), n0) && r.get(Y.data(), n0) && r.get(&rng) && r.get(&arith);
    for (int k = 0; k < 3 && ok; ++k) {
        int32_t L = 0;
        ok = r.get(&L) && L > 0 && L < (1 << 26);
        if (ok) {
            pdf[k].resize((size_t)L);
            ok = r.get(pdf[k].data(), (size_t)L);
        }
    }
    if (ok) {
        data.resize((size_t)xs * ys);
        ok = r.get(data.data(), data.size());
    }
    std::fclose(f);
    if (!ok) { std::fprintf(stderr, "%s: not a bamf_driver rjmcmc input\n", in_path); return 1; }

    const bamf_emitters e0 = {n0, I.data(), X.data(), Y.data(), bg};
    const int64_t steps = (int64_t)p.N_Burnin + p.N_Trials;
    if (steps < 0 || steps > (1 << 24) || p.Grid_Zoom < 0 || p.Grid_Zoom > 64) {
        std::fprintf(stderr, "unreasonable chain length or zoom\n");
        return 1;
    }
    const int ce = (int)steps + 1, cr = ce * BAMF_NMAX;
    struct Buf {
        std::vector<int32_t> N, JT, A, Ix, S;
        std::vector<float> LLR, PR, BG, ABG, BBG, Ph, X, Y;
        bamf_chain c;
    } b[2];
    for (auto &q : b) {
        q.N.resize(ce); q.JT.resize(ce); q.A.resize(ce); q.LLR.resize(ce); q.PR.resize(ce); q.BG.resize(ce);
        q.ABG.resize(ce); q.BBG.resize(ce); q.Ix.resize(cr); q.S.resize(cr); q.Ph.resize(cr); q.X.resize(cr);
        q.Y.resize(cr);
        q.c = bamf_chain{ce, cr, 0, 0, q.N.data(), q.LLR.data(), q.PR.data(), q.JT.data(), q.A.data(), q.BG.data(),
                         q.ABG.data(), q.BBG.data(), q.Ix.data(), q.Ph.data(), q.X.data(), q.Y.data(), q.S.data()};
    }
    const int64_t G = (int64_t)xs * ys * p.Grid_Zoom * p.Grid_Zoom;
    std::vector<float> pg((size_t)G), pb((size_t)G);
    bamf_counters cnt;
    std::memset(&cnt, 0, sizeof cnt);
    const bamf_status st = bamf_crjmcmc_host(data.data(), xs, ys, &e0, &p, pdf[0].data(), (int)pdf[0].size(),
                                             pdf[1].data(), (int)pdf[1].size(), pdf[2].data(), (int)pdf[2].size(),
                                             nullptr, &rng, arith, G ? pg.data() : nullptr, G ? pb.data() : nullptr,
                                             &b[0].c, &b[1].c, &cnt);
    FILE *o = std::fopen(out_path, "wb");
    if (!o) { std::perror(out_path); return 1; }
    std::fwrite("BAMFRO1", 1, 8, o);
    put(o, &st, 1);
    if (st == BAMF_OK) {
        for (auto &q : b) {
            const int32_t ne = q.c.n_entries, nr = q.c.n_records;
            put(o, &ne, 1); put(o, &nr, 1);
            put(o, q.N.data(), ne); put(o, q.LLR.data(), ne); put(o, q.PR.data(), ne); put(o, q.JT.data(), ne);
            put(o, q.A.data(), ne); put(o, q.BG.data(), ne); put(o, q.ABG.data(), ne); put(o, q.BBG.data(), ne);
            put(o, q.Ix.data(), nr); put(o, q.Ph.data(), nr); put(o, q.X.data(), nr); put(o, q.Y.data(), nr);
            put(o, q.S.data(), nr);
        }
        put(o, &G, 1);
        put(o, pg.data(), (size_t)G);
        put(o, pb.data(), (size_t)G);
        put(o, &cnt.N_jump, 30);
    } else {
        std::fprintf(stderr, "bamf_crjmcmc_host: status %d %s\n", st, bamf_last_error());
    }
    std::fclose(o);
    return st == BAMF_OK ? 0 : 1;
}

/* the reference forward model (LibRJMCMC.cpp:15-59) with an erf-integrated
 * Gaussian of width sigma, for the synthetic ROIs */
void model(int side, const std::vector<double> &X, const std::vector<double> &Y, const std::vector<double> &I,
           double bg, double sigma, std::vector<double> &out)
{
    out.assign((size_t)side * side, bg);
    const double c = 1.0 / (std::sqrt(2.0) * sigma);
    for (size_t k = 0; k < X.size(); ++k)
        for (int x = 0; x < side; ++x) {
            const double gx = 0.5 * (std::erf((x + 1 - X[k]) * c) - std::erf((x - X[k]) * c));
            for (int y = 0; y < side; ++y) {
                const double gy = 0.5 * (std::erf((y + 1 - Y[k]) * c) - std::erf((y - Y[k]) * c));
                out[(size_t)y + (size_t)side * x] += I[k] * gx * gy;
            }
        }
}

int run_batch(int n, int jumps, unsigned seed)
{
    if (n < 1 || jumps < 1) return usage();
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const int sides[5] = {8, 12, 16, 20, 24};
    std::vector<float> data, sigma((size_t)n);
    std::vector<int64_t> off((size_t)n);
    std::vector<int32_t> xs((size_t)n), ys((size_t)n);
    double true_n = 0;
    std::vector<double> lam;
    for (int k = 0; k < n; ++k) {
        const int side = sides[(int)(U(g) * 5) % 5];
        const int nk = std::min(24, (int)std::poisson_distribution<int>(12.0 * U(g) + 1e-12)(g));
        std::vector<double> X(nk), Y(nk), I(nk);
        for (int e = 0; e < nk; ++e) {
            X[e] = side * U(g);
            Y[e] = side * U(g);
            I[e] = std::exp(std::log(1000.0) + 0.4 * std::normal_distribution<double>()(g));
        }
        sigma[k] = (float)(1.1 + 0.4 * U(g));
        model(side, X, Y, I, 5.0 + 45.0 * U(g), sigma[k], lam);
        off[k] = (int64_t)data.size();
        xs[k] = ys[k] = side;
        for (double v : lam) data.push_back((float)std::poisson_distribution<long>(v)(g));
        true_n += nk;
    }
    /* priors: SignalPDF the generator's log-normal on 0:10:12000, OffSetPDF
     * a gamma with the mean and variance of U[5,50] (shape 4.48, scale 6.14),
     * BackPDF zeros */
    const int L = 1201;
    std::vector<float> sig(L, 0.0f), offp(L, 0.0f), back(L, 0.0f);
    const double shape = 27.5 * 27.5 / (45.0 * 45.0 / 12.0), scale = (45.0 * 45.0 / 12.0) / 27.5;
    for (int i = 1; i < L; ++i) {
        const double x = 10.0 * i, z = (std::log(x) - std::log(1000.0)) / 0.4;
        sig[i] = (float)(std::exp(-0.5 * z * z) / (x * 0.4 * std::sqrt(2 * 3.14159265358979323846)));
        offp[i] = (float)std::exp((shape - 1) * std::log(x) - x / scale - std::lgamma(shape) - shape * std::log(scale));
    }
    bamf_mcmc_params p;
    std::memset(&p, 0, sizeof p);
    p.PSFsigma = 1.3f; p.N_Burnin = jumps; p.N_Trials = jumps;
    p.I_stdFg = 10.0f; p.I_stdBg = 10.0f; p.X_stdFg = 0.1f; p.X_stdBg = 0.1f;
    const float P[8] = {0.5f, 0.1f, 0.1f, 0.15f, 0.15f, 0.0f, 0.0f, 0.0f};
    std::memcpy(p.P_Burnin, P, sizeof P);
    std::memcpy(p.P_Trials, P, sizeof P);
    p.Rho = 6.0f / 288.0f; p.Bnd_out = 2.0f; p.Grid_Zoom = 20; p.Split_std = 0.5f; p.Icutoff = 0.0f;
    p.BG_std = 1.0f; p.ABBG_std = 0.0f; p.DX = 10.0f;
    p.PSFsize[0] = 10; p.PSFsize[1] = 10; p.PSFsize[2] = 2; p.PSFsize[3] = 2;
    bamf_roi_batch b;
    std::memset(&b, 0, sizeof b);
    b.n_rois = n; b.data = data.data(); b.offsets = off.data(); b.xsize = xs.data(); b.ysize = ys.data();
    /* the empty start's offset: the grid position of the offset prior's
     * maximum (rjmcmc.m:47) */
    int mode = 0;
    for (int i = 1; i < L; ++i)
        if (offp[i] > offp[mode]) mode = i;
    b.psf_sigma = sigma.data(); b.bg0 = 10.0f * (float)mode; b.proposal = BAMF_PROPOSAL_REFERENCE;
    const bamf_priors pri = {offp.data(), L, sig.data(), L, back.data(), L};
    std::vector<int32_t> map_n((size_t)n), status((size_t)n);
    bamf_batch_results res;
    std::memset(&res, 0, sizeof res);
    res.map_n = map_n.data();
    res.status = status.data();
    bamf_workspace *ws = nullptr;
    if (bamf_workspace_create(&ws) != BAMF_OK) return 1;
    bamf_status st = bamf_rjmcmc_batch_host(ws, &b, &p, &pri, 1234u, BAMF_ARITH_FAST, &res); /* warm */
    const auto t0 = std::chrono::steady_clock::now();
    if (st == BAMF_OK) st = bamf_rjmcmc_batch_host(ws, &b, &p, &pri, 1234u, BAMF_ARITH_FAST, &res);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    bamf_workspace_destroy(ws);
    if (st != BAMF_OK) {
        std::fprintf(stderr, "bamf_rjmcmc_batch_host: status %d %s\n", st, bamf_last_error());
        return 1;
    }
    double mn = 0;
    int bad = 0;
    for (int k = 0; k < n; ++k) {
        mn += map_n[k];
        bad += status[k] != BAMF_OK;
    }
    std::printf("{\"n_rois\": %d, \"jumps\": [%d, %d], \"seconds\": %.6f, \"rois_per_s\": %.1f, "
                "\"map_n_mean\": %.4f, \"true_n_mean\": %.4f, \"roi_errors\": %d}\n",
                n, jumps, jumps, secs, n / secs, mn / n, true_n / n, bad);
    return bad ? 1 : 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) return usage();
    const std::string cmd = argv[1];
    if (cmd == "rjmcmc" && argc == 4) return run_rjmcmc(argv[2], argv[3]);
    if (cmd == "batch" && (argc == 4 || argc == 5))
        return run_batch(std::atoi(argv[2]), std::atoi(argv[3]), argc == 5 ? (unsigned)std::atoi(argv[4]) : 1u);
    return usage();
}
