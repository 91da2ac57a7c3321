"""The fast (production) sampler against the reference's posterior on the
batched uneven workload: ROI sides 8..24 px, emitter counts Poisson(lambda)
with lambda up to 12, PSF sigma 1.1..1.5 px, backgrounds 5..50.

Fast arithmetic does not follow the reference chain path by path (hardware
math, incremental model, move types shared by the 8 chains of a slot group),
so it is checked in distribution against the oracle (the C restatement,
bit-identical to the reference build): after the same number of jumps from
the same start, a chain of either sampler is a draw from the same law.
"""
import concurrent.futures as cf

import numpy as np
import pytest
from scipy.stats import chi2_contingency, combine_pvalues, ks_2samp

from bamf_gb300 import rjstruct, sampler, synth

pytestmark = pytest.mark.gpu

SIDES = (8, 12, 16, 20, 24)
PER_SIDE = 8          # ROIs per side: one copy of each in every slot group of 8
GPU_COPIES = 1024     # GPU chains per ROI
ORACLE_CHAINS = 384   # oracle chains per ROI
JUMPS = 1000          # burn-in and trial jumps per chain


def _pick_rois(seed=31):
    """PER_SIDE ROIs of every side from the uneven generator, spread over
    the emitter counts the generator made for that side (lambda ~ U[0, 12]),
    up to 18 true emitters."""
    b = synth.roi_batch_uneven(600, seed=seed)
    picked = []
    for s in SIDES:
        ks = np.flatnonzero((b.xsize == s) & (b.true_n <= 18))
        ks = ks[np.argsort(b.true_n[ks], kind="stable")]
        picked.extend(int(ks[int(round(q))]) for q in np.linspace(0, len(ks) - 1, PER_SIDE))
    return b, picked


def _oracle_finals(oracle_port, roi, params, rj, bg0, n_chains, seed):
    args = (params, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)

    def one(c):
        r = oracle_port.run_chain("port_native", roi, *args, e0=([], [], [], bg0), rng=(seed, c, 0))
        ch = r["chain"]
        n, I, X, Y, S = sampler._emitters_of(ch, len(ch["N"]) - 1)
        nn = int(ch["N"][-1])
        return nn, X[:nn].astype(np.float64), Y[:nn].astype(np.float64), int(r["chain_test"]["N"].max())

    with cf.ThreadPoolExecutor(16) as ex:
        return list(ex.map(one, range(n_chains)))


def _tv(a, b, K):
    ha = np.bincount(a, minlength=K) / len(a)
    hb = np.bincount(b, minlength=K) / len(b)
    return 0.5 * np.abs(ha - hb).sum()


def _tv_permutation_p(a, b, n_perm=2000, seed=0):
    """Share of label permutations of the pooled counts whose total
    variation is at least the observed one (the TV's own null distribution:
    a count posterior spread over many values has a larger TV between two
    finite samples of the same law)."""
    K = int(max(a.max(), b.max())) + 1
    obs = _tv(a, b, K)
    pool = np.concatenate([a, b])
    rng = np.random.default_rng(seed)
    ge = 0
    for _ in range(n_perm):
        q = rng.permutation(pool)
        ge += _tv(q[:len(a)], q[len(a):], K) >= obs - 1e-12
    return (ge + 1) / (n_perm + 1)


def _count_test(a, b):
    """Chi-square test of homogeneity of two count samples (bins with too few
    expected counts merged into their neighbour) and the total variation."""
    K = int(max(a.max(), b.max())) + 1
    ha = np.bincount(a, minlength=K).astype(float)
    hb = np.bincount(b, minlength=K).astype(float)
    tv = _tv(a, b, K)
    tab = [[0.0, 0.0]]
    for i in range(K):
        if min(tab[-1]) >= 10 and tab[-1][0] + tab[-1][1] >= 20:
            tab.append([0.0, 0.0])
        tab[-1][0] += ha[i]
        tab[-1][1] += hb[i]
    if len(tab) > 1 and min(tab[-1]) < 10:
        last = tab.pop()
        tab[-1][0] += last[0]
        tab[-1][1] += last[1]
    if len(tab) < 2:
        return 1.0, tv
    return float(chi2_contingency(np.array(tab).T)[1]), tv


def test_fast_sampler_matches_the_reference_posterior_per_size_class(cuda_lib, oracle_port):
    """Per size class (sides 8, 12, 16, 20, 24; 8 ROIs each, emitter counts
    spanning what lambda in [0, 12] gives), the final states of 1024
    independent fast GPU chains and of 384 oracle chains per ROI after
    1000 + 1000 jumps agree: the emitter-count distributions (chi-square
    homogeneity test, total variation), the per-chain mean X and mean Y
    (two-sample KS; one value per chain, so the samples are independent)
    and the pooled emitter positions (KS).  Each slot group of 8 GPU chains
    holds one copy of each ROI of a side, so no two GPU chains of one ROI
    share a move stream.

    A GPU chain state holds at most BAMF_NMAX = 32 emitters (a proposal
    beyond is rejected and counted in `overflow`); the reference's has no
    limit, and its early chains on large crowded ROIs do propose more than 32
    (the reference birth ratio overfits in burn-in).  A ROI where a GPU chain
    overflowed or an oracle chain proposed 32 or more emitters is left out of
    the comparison; at least 30 of the 40 must remain."""
    b, picked = _pick_rois()
    rj = rjstruct.uneven_rjstruct()
    rj.N_Burnin = rj.N_Trials = JUMPS
    bg0 = rjstruct.initial_bg(rj)
    # GPU: ROIs of one side interleaved, copy by copy
    order = [picked[i * PER_SIDE + j] for i in range(len(SIDES)) for _ in range(GPU_COPIES) for j in range(PER_SIDE)]
    big = synth._pack([b.roi(k) for k in order], [b.sigma[k] for k in order], [b.bg[k] for k in order],
                      [b.true_n[k] for k in order], [b.true_x[k] for k in order], [b.true_y[k] for k in order],
                      [b.true_i[k] for k in order])
    p = rjstruct.mcmc_params(rj)
    got = sampler.Sampler().run_host(big, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=101,
                                     arith="fast", bg0=bg0)
    assert (got["status"] == 0).all()
    fs, fn = got["final_state"], got["final_n"]
    nmax = (fs.shape[1] - 4) // 4
    order = np.array(order)
    rows = []
    pvals = {"count": [], "tv": [], "mx": [], "my": [], "x": [], "y": []}
    left_out = []
    for k in picked:
        idx = np.flatnonzero(order == k)
        if got["overflow"][idx].any():
            left_out.append((int(b.xsize[k]), int(b.true_n[k]), "gpu overflow"))
            continue
        gn = fn[idx]
        gx = [fs[i, 4 + nmax:4 + nmax + fn[i]].astype(np.float64) for i in idx]
        gy = [fs[i, 4 + 2 * nmax:4 + 2 * nmax + fn[i]].astype(np.float64) for i in idx]
        pk = rjstruct.mcmc_params(rj)
        pk.PSFsigma = float(b.sigma[k])
        ora = _oracle_finals(oracle_port, b.roi(k), pk, rj, bg0, ORACLE_CHAINS, seed=500 + k)
        on = np.array([o[0] for o in ora])
        if max(o[3] for o in ora) >= 32:
            left_out.append((int(b.xsize[k]), int(b.true_n[k]), "oracle proposed >= 32"))
            continue
        pc, tv = _count_test(gn, on)
        ptv = _tv_permutation_p(gn, on)
        gmx = np.array([x.mean() for x in gx if x.size]); omx = np.array([o[1].mean() for o in ora if o[1].size])
        gmy = np.array([y.mean() for y in gy if y.size]); omy = np.array([o[2].mean() for o in ora if o[2].size])
        pmx = ks_2samp(gmx, omx).pvalue if gmx.size > 20 and omx.size > 20 else 1.0
        pmy = ks_2samp(gmy, omy).pvalue if gmy.size > 20 and omy.size > 20 else 1.0
        gxa, oxa = np.concatenate(gx), np.concatenate([o[1] for o in ora])
        gya, oya = np.concatenate(gy), np.concatenate([o[2] for o in ora])
        px = ks_2samp(gxa, oxa).pvalue if gxa.size > 20 and oxa.size > 20 else 1.0
        py = ks_2samp(gya, oya).pvalue if gya.size > 20 and oya.size > 20 else 1.0
        for key, v in (("count", pc), ("tv", ptv), ("mx", pmx), ("my", pmy), ("x", px), ("y", py)):
            pvals[key].append(v)
        rows.append((int(b.xsize[k]), int(b.true_n[k]), float(gn.mean()), float(on.mean()), tv, pc, pmx, pmy, px, py))
    for r in rows:
        print("side %2d true N %2d | mean N gpu %5.2f oracle %5.2f | TV %.3f | p count %.3f meanX %.3f "
              "meanY %.3f X %.3f Y %.3f" % r)
    print("left out (side, true N, why):", left_out)
    assert len(rows) >= 30, left_out
    tvs = np.array([r[4] for r in rows])
    comb = {k: combine_pvalues(v, method="fisher")[1] for k, v in pvals.items()}
    print("max TV %.3f, mean TV %.3f; Fisher-combined p:" % (tvs.max(), tvs.mean()), comb)
    # about 200 tests at 1e-4 each (the TV permutation test at its 2000-draw
    # resolution, 5e-4): a family-wise false alarm rate of a few per cent
    for key, v in pvals.items():
        assert min(v) > (4e-4 if key == "tv" else 1e-4), (key, min(v))
        assert comb[key] > 1e-3, (key, comb[key])
    # measured on a GB300: mean TV 0.031 over 35 ROIs, largest 0.12 on a ROI
    # whose count posterior spreads over ~10 values (its permutation p 0.02)
    assert tvs.mean() < 0.05, tvs.mean()
    # the counts moved away from the empty start, so the test has power
    assert np.mean([r[2] for r in rows]) > 2.0


def test_fast_map_counts_agree_with_the_oracle_like_two_oracle_runs(cuda_lib, oracle_port):
    """MAP emitter counts (findMap.m:29-45) of 1200 uneven ROIs at the full
    3000 + 3000 jumps: the fast GPU sampler agrees with an oracle run as
    often as two oracle runs with independent streams agree with each
    other, and its mean MAP count is the oracle's."""
    b = synth.roi_batch_uneven(1200, seed=43)
    rj = rjstruct.uneven_rjstruct()
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    oa = oracle_port.run_batch(b, *args, bg0, seed=1, threads=16, kind="port_native")["map_n"]
    ob = oracle_port.run_batch(b, *args, bg0, seed=2, threads=16, kind="port_native")["map_n"]
    s = sampler.Sampler()
    fa = s.run_host(b, *args, seed=3, arith="fast", bg0=bg0)
    fb = s.run_host(b, *args, seed=4, arith="fast", bg0=bg0)
    assert (fa["status"] == 0).all() and (fb["status"] == 0).all()
    fa, fb = fa["map_n"], fb["map_n"]
    a_oo = np.mean(oa == ob)
    a_fo = 0.5 * (np.mean(fa == oa) + np.mean(fb == ob))
    a_ff = np.mean(fa == fb)
    print(f"MAP agreement oracle/oracle {a_oo:.3f}, fast/oracle {a_fo:.3f}, fast/fast {a_ff:.3f}; "
          f"mean MAP oracle {oa.mean():.3f} {ob.mean():.3f} fast {fa.mean():.3f} {fb.mean():.3f}; "
          f"true {b.true_n.mean():.3f}")
    assert abs(a_fo - a_oo) < 0.04, (a_fo, a_oo)
    assert abs(a_ff - a_oo) < 0.04, (a_ff, a_oo)
    assert abs(0.5 * (fa.mean() + fb.mean()) - 0.5 * (oa.mean() + ob.mean())) < 0.08
    # per size class too
    for s_ in SIDES:
        m = b.xsize == s_
        d = 0.5 * (fa[m].mean() + fb[m].mean()) - 0.5 * (oa[m].mean() + ob[m].mean())
        assert abs(d) < 0.25, (s_, d)


def test_incremental_model_drift_is_bounded(cuda_lib):
    """Fast arithmetic updates the model image incrementally (M' = M - old
    stencils + new) and rebuilds it from the state every 512 jumps.  Just
    before each rebuild the incrementally kept image differs from the
    rebuilt one by a small relative amount on every ROI of an uneven batch
    (float rounding of ~500 updates), so the likelihood ratios the chain
    accepts on are those of its state."""
    b = synth.roi_batch_uneven(3000, seed=47)
    rj = rjstruct.uneven_rjstruct()
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    r = sampler.Sampler().run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=8, arith="fast",
                                   bg0=bg0, model_drift=True)
    assert (r["status"] == 0).all()
    d = r["model_drift"]
    print("relative model drift before rebuilds: max %.3g, 99th pct %.3g, median %.3g"
          % (d.max(), np.percentile(d, 99), np.median(d)))
    assert np.isfinite(d).all() and (d >= 0).all()
    assert (d > 0).mean() > 0.5          # the measurement ran (6000 jumps: 11 rebuilds per chain)
    # measured on a GB300: max 2.6e-6, median 9.6e-7 (float rounding of
    # model values up to ~1e3, a few ulp after ~500 updates)
    assert d.max() < 2e-5, d.max()
    assert np.median(d) < 5e-6, np.median(d)
