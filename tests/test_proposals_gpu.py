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
