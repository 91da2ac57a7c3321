"""MAP emitter sets (findMap) and fixed-count refinement (mcmc) on the GPU:
the device summaries against the numpy restatement on the same thinned
chain records, and the localisation they give against the generator's
truth."""
import numpy as np
import pytest

from bamf_gb300 import mapfit, rjstruct, synth
from oracle import mapfit_port

pytestmark = pytest.mark.gpu


def _dev(b):
    import torch
    d = {k: torch.from_numpy(v).cuda() for k, v in
         (("data", b.data), ("offsets", b.offsets), ("xsize", b.xsize), ("ysize", b.ysize))}
    d["side_max"] = int(max(b.xsize.max(), b.ysize.max()))
    return d


def test_map_kmeans_and_refine_match_restatement_and_truth(cuda_lib):
    import torch
    from scipy.optimize import linear_sum_assignment
    from bamf_gb300 import sampler
    b = synth.roi_batch_c0(120, seed=3)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = 1500
    rj.N_BurninMCMC = rj.N_TrialsMCMC = 1000
    dev = _dev(b)
    s = sampler.Sampler()
    p = rjstruct.mcmc_params(rj)
    outs, thin = mapfit._run(s, dev, p, rj, 11, "fast", "reference", 200, rjstruct.initial_bg(rj))
    km = mapfit.map_kmeans(outs["pos_trace"], thin, outs["n_entries"], outs["map_n"]).cpu().numpy()
    recs = outs["pos_trace"].cpu().numpy()
    ne = outs["n_entries"].cpu().numpy()
    mn = outs["map_n"].cpu().numpy()
    for r in range(b.n):
        ref = mapfit_port.map_kmeans(recs[r], thin, ne[r], mn[r])
        got = mapfit.unpack(km[r:r + 1])
        assert got["N"][0] == ref["N"] and got["records"][0] == ref["records"]
        np.testing.assert_allclose(got["Bg"][0], ref["Bg"], rtol=1e-5)
        for name in ("X", "Y", "I", "X_SE", "Y_SE", "I_SE"):
            np.testing.assert_allclose(got[name][0], ref[name], rtol=2e-4, atol=2e-5, equal_nan=True,
                                       err_msg=f"roi {r} {name}")
    # refinement statistics against the restatement
    res = mapfit.analyze(dev, rj, seed=11, pos_len=200, s=s)
    np.testing.assert_array_equal(res["map"]["N"], mn)
    # localisation against the truth: Hungarian matching on ROIs whose MAP
    # count is right; RMSE of the pairs within 1 px (emitters closer than the
    # PSF can be fitted as one plus a split of another: the count matches
    # but such pairs are not localisations) and the fraction matched
    def rmse_of(which):
        se, cnt, ok, tot = 0.0, 0, 0, 0
        for r in range(b.n):
            k = int(b.true_n[r])
            if k == 0 or res["map"]["N"][r] != k:
                continue
            ok += 1
            X, Y = res[which]["X"][r, :k], res[which]["Y"][r, :k]
            d2 = (X[:, None] - b.true_x[r][None, :]) ** 2 + (Y[:, None] - b.true_y[r][None, :]) ** 2
            i, j = linear_sum_assignment(d2)
            m = d2[i, j] < 1.0
            se += d2[i, j][m].sum()
            cnt += int(m.sum())
            tot += k
        return ok, np.sqrt(se / cnt), cnt / tot
    ok, rk, fk = rmse_of("map")
    _, rr, fr = rmse_of("refined")
    for r in range(3):
        print("roi", r, "truth", np.round(b.true_x[r], 2), np.round(b.true_y[r], 2),
              "kmeans", np.round(res["map"]["X"][r, :4], 2), np.round(res["map"]["Y"][r, :4], 2),
              "refined", np.round(res["refined"]["X"][r, :4], 2), np.round(res["refined"]["Y"][r, :4], 2),
              "N", res["map"]["N"][r], res["refined"]["N"][r])
    print("ROIs with the right MAP count:", ok, "RMSE (px) k-means", rk, "refined", rr,
          "matched within 1 px", fk, fr)
    assert ok > 60 and rk < 0.25 and rr < 0.2 and rr <= 1.1 * rk and fk > 0.9 and fr > 0.9


def test_refine_stats_match_restatement(cuda_lib):
    import torch
    from bamf_gb300 import sampler
    b = synth.roi_batch_c0(40, seed=5)
    rj = rjstruct.c0_rjstruct()
    rj.N_BurninMCMC = rj.N_TrialsMCMC = 800
    dev = _dev(b)
    n = b.n
    k = np.maximum(b.true_n, 1).astype(np.int32)
    ixy = np.zeros((n, 3, 32), np.float32)
    for r in range(n):
        m = int(b.true_n[r])
        ixy[r, 0, :m] = 1000.0
        ixy[r, 1, :m] = b.true_x[r]
        ixy[r, 2, :m] = b.true_y[r]
        if m == 0:
            ixy[r, :, 0] = (1000.0, 8.0, 8.0)
    dev["init_n"] = torch.from_numpy(k).cuda()
    dev["init_ixy"] = torch.from_numpy(ixy).cuda()
    s = sampler.Sampler()
    outs, thin = mapfit._run(s, dev, rjstruct.refine_params(rj), rj, 3, "fast", "reference", 100,
                             rjstruct.initial_bg(rj))
    rs = mapfit.refine_stats(outs["pos_trace"], thin, outs["n_entries"]).cpu().numpy()
    recs = outs["pos_trace"].cpu().numpy()
    ne = outs["n_entries"].cpu().numpy()
    for r in range(n):
        ref = mapfit_port.refine_stats(recs[r], thin, ne[r])
        got = mapfit.unpack(rs[r:r + 1])
        assert got["N"][0] == ref["N"] == k[r]
        for name in ("X", "Y", "I", "X_SE", "Y_SE", "I_SE"):
            np.testing.assert_allclose(got[name][0], ref[name], rtol=1e-5, atol=1e-6, equal_nan=True)
