"""Birth proposals of the fast batched sampler (UNIFORM and LEARNED) and the
chain traces used for effective-sample-size measurement."""
import numpy as np
import pytest

from bamf_gb300 import proposal, rjstruct, sampler, synth

pytestmark = pytest.mark.gpu


def _c0(n_rois, steps, seed=0):
    b = synth.roi_batch_c0(n_rois, seed=seed)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = steps
    return b, rj, rjstruct.mcmc_params(rj), rjstruct.initial_bg(rj)


def _replicate(b, k, copies):
    """A batch of `copies` copies of ROI k (independent chains, one posterior)."""
    roi = b.roi(k)
    return synth._pack([roi] * copies, [b.sigma[k]] * copies, [b.bg[k]] * copies,
                       [b.true_n[k]] * copies, [b.true_x[k]] * copies, [b.true_y[k]] * copies,
                       [b.true_i[k]] * copies)


def _second_half(tr, n_entries):
    out = []
    for i in range(tr.shape[0]):
        e = min(int(n_entries[i]), tr.shape[1])
        out.append(tr[i, e // 2:e])
    return np.concatenate(out)


def _hist(v, K=12):
    h = np.bincount(np.minimum(v.astype(np.int64), K - 1), minlength=K).astype(float)
    return h / h.sum()


def test_uniform_proposal_recovers_emitter_counts(cuda_lib):
    b, rj, p, bg0 = _c0(200, 3000)
    s = sampler.Sampler()
    ref = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1, arith="fast", bg0=bg0)
    uni = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1, arith="fast", bg0=bg0,
                     proposal="uniform")
    assert (uni["status"] == 0).all() and (uni["overflow"] == 0).all()
    err_ref = np.mean(np.abs(ref["map_n"] - b.true_n))
    err_uni = np.mean(np.abs(uni["map_n"] - b.true_n))
    print("MAP |N - truth|: reference proposal", err_ref, "uniform", err_uni)
    assert err_uni <= err_ref + 0.3
    assert np.mean(uni["map_n"] == b.true_n) > 0.5


def test_traces_agree_with_map_count_and_state(cuda_lib):
    b, rj, p, bg0 = _c0(64, 600)
    s = sampler.Sampler()
    T = 2 * 600
    a = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=4, arith="fast", bg0=bg0,
                   proposal="uniform", trace_len=T)
    c = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=4, arith="fast", bg0=bg0,
                   proposal="uniform")
    # map_n from the caller's trace equals map_n from the internal one
    np.testing.assert_array_equal(a["map_n"], c["map_n"])
    for i in range(b.n):
        e = int(a["n_entries"][i])
        assert 0 < e <= T
        nt, xt = a["n_trace"][i, :e], a["x_trace"][i, :e]
        np.testing.assert_array_equal(np.isnan(xt), nt == 0)
        assert (a["n_trace"][i, e:] == 0).all()
        ok = np.isfinite(xt)
        assert ((xt[ok] >= -10) & (xt[ok] <= 26)).all()
        # last entry: the final state's count (placeholder entry counts 0)
        assert nt[-1] == a["final_n"][i] or a["final_n"][i] == 0


def _learned_tables(b, cells_fn):
    maps = [cells_fn(i, int(b.xsize[i]), int(b.ysize[i])) for i in range(b.n)]
    return proposal.batch_tables(maps, b.xsize, b.ysize)


def test_learned_proposal_leaves_the_posterior_unchanged(cuda_lib):
    """An arbitrary (badly placed) learned birth density must not move the
    posterior: the pooled emitter-count and mean-X distributions of 384
    chains on one ROI agree with the UNIFORM proposal's."""
    b0, rj, p, bg0 = _c0(8, 2500)
    b = _replicate(b0, 1, 384)
    rng = np.random.default_rng(11)
    X, Y = int(b.xsize[0]), int(b.ysize[0])
    bad = rng.gamma(0.2, size=(4 * X, 4 * Y))       # spiky, unrelated to the data
    cdf, sub = _learned_tables(b, lambda i, X, Y: bad)
    s = sampler.Sampler()
    T = 5000
    kw = dict(arith="fast", bg0=bg0, trace_len=T)
    uni = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=21, proposal="uniform", **kw)
    lea = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=22, proposal="learned",
                     birth=(cdf, sub), **kw)
    assert (lea["status"] == 0).all()
    nu = _second_half(uni["n_trace"], uni["n_entries"])
    nl = _second_half(lea["n_trace"], lea["n_entries"])
    hu, hl = _hist(nu), _hist(nl)
    tv = 0.5 * np.abs(hu - hl).sum()
    print("true N", b.true_n[0], "uniform", np.round(hu[:8], 3), "learned", np.round(hl[:8], 3), "TV", tv)
    assert tv < 0.05
    xu = _second_half(uni["x_trace"], uni["n_entries"])
    xl = _second_half(lea["x_trace"], lea["n_entries"])
    mu, ml = np.nanmean(xu), np.nanmean(xl)
    print("mean X", mu, ml)
    assert abs(mu - ml) < 0.15


def test_learned_proposal_with_a_good_density_converges_faster(cuda_lib):
    """A density concentrated at the true emitters puts births where the data
    want them: from an empty start, short chains reach the right emitter
    count on more ROIs than with UNIFORM births."""
    b, rj, p, bg0 = _c0(200, 150)

    def truth_cells(i, X, Y):
        cx = (np.arange(4 * X) + 0.5) / 4
        cy = (np.arange(4 * Y) + 0.5) / 4
        g = np.full((4 * X, 4 * Y), 1e-3)
        for x, y in zip(b.true_x[i], b.true_y[i]):
            g += np.exp(-((cx[:, None] - x) ** 2 + (cy[None, :] - y) ** 2) / (2 * 0.3 ** 2))
        return g

    cdf, sub = _learned_tables(b, truth_cells)
    s = sampler.Sampler()
    uni = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=5, arith="fast", bg0=bg0,
                     proposal="uniform")
    lea = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=5, arith="fast", bg0=bg0,
                     proposal="learned", birth=(cdf, sub))
    eu = np.mean(uni["map_n"] == b.true_n)
    el = np.mean(lea["map_n"] == b.true_n)
    print("MAP count right after 150+150 jumps: uniform", eu, "learned", el)
    assert el > eu + 0.1


def test_learned_split_leaves_the_posterior_unchanged(cuda_lib):
    """Split-heavy chains (split and merge half of all moves): with LEARNED
    proposals half of the splits place the first emitter from the learned
    density and the split/merge ratios carry the offset's mixture density.
    With an arbitrary spiky density the pooled emitter-count and mean-X
    distributions of 384 chains on one ROI agree with UNIFORM's."""
    b0, rj, _, bg0 = _c0(8, 2500, seed=4)
    P = [0.3, 0.25, 0.25, 0.1, 0.1, 0.0, 0.0, 0.0]
    rj.P_Burnin = rj.P_Trials = P
    p = rjstruct.mcmc_params(rj)
    k = int(np.argmax(b0.true_n))
    b = _replicate(b0, k, 384)
    rng = np.random.default_rng(5)
    X, Y = int(b.xsize[0]), int(b.ysize[0])
    bad = rng.gamma(0.2, size=(4 * X, 4 * Y))
    cdf, sub = _learned_tables(b, lambda i, X, Y: bad)
    s = sampler.Sampler()
    kw = dict(arith="fast", bg0=bg0, trace_len=5000)
    uni = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=31, proposal="uniform", **kw)
    lea = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=32, proposal="learned",
                     birth=(cdf, sub), **kw)
    assert (lea["status"] == 0).all() and (uni["status"] == 0).all()
    hu = _hist(_second_half(uni["n_trace"], uni["n_entries"]))
    hl = _hist(_second_half(lea["n_trace"], lea["n_entries"]))
    tv = 0.5 * np.abs(hu - hl).sum()
    print("true N", b.true_n[0], "uniform", np.round(hu[:8], 3), "learned", np.round(hl[:8], 3), "TV", tv)
    assert tv < 0.05
    mu = np.nanmean(_second_half(uni["x_trace"], uni["n_entries"]))
    ml = np.nanmean(_second_half(lea["x_trace"], lea["n_entries"]))
    assert abs(mu - ml) < 0.15


def test_learned_split_separates_a_merged_pair_faster(cuda_lib):
    """ROIs with two emitters 2.5-3.5 px apart (5-7 Split_std), each chain
    started from one emitter at their intensity-weighted mean, and only
    jumps, splits and merges: with a density concentrated at the true
    emitters, LEARNED splits reach the right count on more ROIs within
    100+100 jumps than Gaussian splits alone.  (At 1.2-1.8 px, within reach
    of the Gaussian offsets, both find the pair on ~0.81 of ROIs.)"""
    rng = np.random.default_rng(8)
    n = 800
    rois, sig, bgs, tn, tx, ty, ti = [], [], [], [], [], [], []
    for _ in range(n):
        c = rng.uniform(5, 11, 2)
        a = rng.uniform(0, np.pi)
        d = rng.uniform(2.5, 3.5)
        X = np.array([c[0] - 0.5 * d * np.cos(a), c[0] + 0.5 * d * np.cos(a)])
        Y = np.array([c[1] - 0.5 * d * np.sin(a), c[1] + 0.5 * d * np.sin(a)])
        I = rng.lognormal(np.log(1500.0), 0.2, 2)
        lam = synth.model_image(16, 16, X, Y, I, 10.0, 1.3)
        rois.append(rng.poisson(lam).astype(np.float32))
        sig.append(1.3); bgs.append(10.0); tn.append(2); tx.append(X); ty.append(Y); ti.append(I)
    b = synth._pack(rois, sig, bgs, tn, tx, ty, ti)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = 100
    rj.P_Burnin = rj.P_Trials = [0.4, 0.3, 0.3, 0.0, 0.0, 0.0, 0.0, 0.0]
    p = rjstruct.mcmc_params(rj)
    ixy = np.zeros((n, 3, 32), np.float32)
    for i in range(n):
        I = b.true_i[i]
        ixy[i, 0, 0] = I.sum()
        ixy[i, 1, 0] = (I * b.true_x[i]).sum() / I.sum()
        ixy[i, 2, 0] = (I * b.true_y[i]).sum() / I.sum()
    init = {"n": np.ones(n, np.int32), "bg": np.full(n, 10.0, np.float32), "ixy": ixy}

    def truth_cells(i, X, Y):
        cx = (np.arange(4 * X) + 0.5) / 4
        cy = (np.arange(4 * Y) + 0.5) / 4
        g = np.full((4 * X, 4 * Y), 1e-3)
        for x, y in zip(b.true_x[i], b.true_y[i]):
            g += np.exp(-((cx[:, None] - x) ** 2 + (cy[None, :] - y) ** 2) / (2 * 0.3 ** 2))
        return g

    cdf, sub = _learned_tables(b, truth_cells)
    s = sampler.Sampler()
    kw = dict(arith="fast", bg0=10.0, init=init)
    uni = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=3, proposal="uniform", **kw)
    lea = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=3, proposal="learned",
                     birth=(cdf, sub), **kw)
    eu, el = np.mean(uni["final_n"] == 2), np.mean(lea["final_n"] == 2)
    print("two emitters found after 100+100 jumps: gaussian splits", eu, "learned splits", el)
    assert el > eu + 0.1
