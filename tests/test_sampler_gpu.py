"""GPU parity of the sampler against the CPU oracle (the C restatement of
source/c/LibRJMCMC.cpp, itself pinned to the reference build).

Exact arithmetic must reproduce the oracle chain bit for bit: every chain
entry (N, LLR, PR, JumpType, Accepted, BG, ABG, BBG), every emitter record,
the posterior grids and the 30 counters."""
import hashlib
import os

import numpy as np
import pytest

from bamf_gb300 import rjstruct, sampler, synth

pytestmark = pytest.mark.gpu


def _c0(n_rois, steps=None, seed=0):
    b = synth.roi_batch_c0(n_rois, seed=seed)
    rj = rjstruct.c0_rjstruct()
    if steps is not None:
        rj.N_Burnin = rj.N_Trials = steps
    return b, rj


def _bits(a):
    a = np.asarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_same_chain(got, ref):
    for w in ("chain", "chain_test"):
        for f, v in ref[w].items():
            g = got[w][f]
            assert g.shape == v.shape, (w, f, g.shape, v.shape)
            bad = np.flatnonzero(_bits(g) != _bits(v))
            assert bad.size == 0, f"{w}.{f} first mismatch at {bad[0]}: {g[bad[0]]} vs {v[bad[0]]}"
    np.testing.assert_array_equal(got["pgrid"], ref["pgrid"])
    np.testing.assert_array_equal(got["pback"], ref["pback"])
    assert got["counters"] == ref["counters"]


GOLD_C0 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rjmcmc_ref_c0.npz")


def _digest(res):
    """SHA-256 over Chain, Chain_Test, PGrid and PBack in the layout the
    golden fixture hashed (tests/golden/make_rjmcmc_golden.py)."""
    h = hashlib.sha256()
    for w in ("chain", "chain_test"):
        for k in sorted(res[w]):
            h.update(k.encode())
            h.update(np.ascontiguousarray(res[w][k]).tobytes())
    h.update(np.ascontiguousarray(res["pgrid"]).tobytes())
    h.update(np.ascontiguousarray(res["pback"]).tobytes())
    return h.hexdigest()


def test_exact_c0_reproduces_the_reference_build_on_all_200_rois(cuda_lib):
    """The whole plain-RJMCMC workload (200 ROIs of 16x16, 3000 burn-in +
    3000 trial jumps, seed 0 data, uniform stream seed 7 with chain id = ROI
    index) through the exact GPU sampler, compared directly with the golden
    fixture made from the reference sampler compiled unmodified (parity-math
    build): every ROI's Chain and Chain_Test vectors, PGrid and PBack hash to
    the reference's, and its chain length, record count, uniforms drawn and
    30 counters are the reference's."""
    gold = np.load(GOLD_C0)
    n = int(gold["n_rois"])
    b, rj = _c0(n)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    names = [str(x) for x in gold["counter_names"]]
    bad = []
    for start in range(0, n, 50):
        ks = list(range(start, min(n, start + 50)))
        res = sampler.crjmcmc_batch_raw([b.roi(k) for k in ks], p, rj.P_Offset, rj.P_EmPhotons,
                                        rj.P_BgEmPhotons, e0s=[([], [], [], bg0)] * len(ks),
                                        seed=int(gold["seed"]), chain_ids=ks, arith="exact",
                                        records_per_entry=10)
        for k, r in zip(ks, res):
            same = (len(r["chain"]["N"]) == gold["pm_entries"][k]
                    and len(r["chain"]["Index"]) == gold["pm_records"][k]
                    and r["uniforms_used"] == gold["pm_uniforms"][k]
                    and [r["counters"][c] for c in names] == list(gold["pm_counters"][k])
                    and _digest(r) == gold["pm_sha256"][k])
            if not same:
                bad.append(k)
    assert not bad, f"ROIs whose GPU outputs differ from the reference build: {bad[:10]} ({len(bad)} of {n})"


@pytest.mark.parametrize("k", [0, 1, 2, 7])
def test_exact_chain_matches_oracle(cuda_lib, oracle_port, k):
    b, rj = _c0(8, steps=1500)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    ref = oracle_port.run_chain("port", b.roi(k), *args, e0=([], [], [], bg0), rng=(11, k, 0))
    got = sampler.crjmcmc_raw(b.roi(k), *args, e0=([], [], [], bg0), rng=(11, k, 0), arith="exact")
    assert_same_chain(got, ref)


def test_exact_chain_with_start_state(cuda_lib, oracle_port):
    """A start state with emitters, drift and a nonzero rng offset (the
    fixed-N refinement call of mcmc.m:142 uses P = [1 0 ... 0])."""
    b, rj = _c0(4, steps=800, seed=3)
    p = rjstruct.refine_params(rj, drift_x=0.25, drift_y=-0.5)
    k = 1
    X = b.true_x[k].astype(np.float32)
    Y = b.true_y[k].astype(np.float32)
    I = b.true_i[k].astype(np.float32)
    e0 = (I, X, Y, 9.5)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    ref = oracle_port.run_chain("port", b.roi(k), *args, e0=e0, rng=(5, 99, 37))
    got = sampler.crjmcmc_raw(b.roi(k), *args, e0=e0, rng=(5, 99, 37), arith="exact")
    assert_same_chain(got, ref)


def test_exact_batch_matches_oracle(cuda_lib, oracle_port):
    """Batch path: final emitter count, MAP count and counters of every ROI."""
    b, rj = _c0(48, steps=1000)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    ref = oracle_port.run_batch(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, bg0, seed=21,
                                threads=8, kind="port")
    s = sampler.Sampler()
    got = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=21, arith="exact", bg0=bg0)
    assert (got["status"] == 0).all()
    np.testing.assert_array_equal(got["final_n"], ref["final_n"])
    np.testing.assert_array_equal(got["map_n"], ref["map_n"])
    acc = got["counters"][:, 5:10].sum(axis=1)
    np.testing.assert_array_equal(acc, ref["n_accepted"])


def test_fast_batch_runs_and_agrees_in_distribution(cuda_lib):
    """Fast arithmetic draws each jump's move type from a stream shared by the
    chains of a CTA, so its chains do not follow the exact chains path by
    path; each chain's law is the same, so MAP counts, proposal mix and
    acceptance rates agree in distribution."""
    b, rj = _c0(256, steps=1500)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    s = sampler.Sampler()
    ex = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=3, arith="exact", bg0=bg0)
    fa = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=3, arith="fast", bg0=bg0)
    assert (fa["status"] == 0).all() and (fa["overflow"] == 0).all()
    # the MAP count is set by the data: both arithmetics find the same one on most ROIs
    agree = np.mean(fa["map_n"] == ex["map_n"])
    assert agree > 0.6, agree
    assert abs(fa["map_n"].mean() - ex["map_n"].mean()) < 0.3
    assert abs(fa["map_n"].mean() - b.true_n.mean()) < 1.0
    # proposal mix: the move-type frequencies follow P_Burnin / P_Trials in both
    nf = fa["counters"][:, 0:5].sum(axis=0).astype(float)
    ne = ex["counters"][:, 0:5].sum(axis=0).astype(float)
    np.testing.assert_allclose(nf / nf.sum(), ne / ne.sum(), atol=0.01)
    # acceptance rate per move type within a few points
    af = fa["counters"][:, 5:10].sum(axis=0) / nf
    ae = ex["counters"][:, 5:10].sum(axis=0) / ne
    np.testing.assert_allclose(af, ae, atol=0.04)

def test_fast_batch_is_deterministic(cuda_lib):
    """The same seed gives the same chains on every call: the size-class order
    of the ROIs (and so which chains share a move stream) is a stable sort."""
    b, rj = _c0(200, steps=400)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    s = sampler.Sampler()
    r1 = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=5, arith="fast", bg0=bg0)
    r2 = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=5, arith="fast", bg0=bg0)
    for k in ("map_n", "final_n", "final_state", "counters"):
        np.testing.assert_array_equal(r1[k], r2[k], err_msg=k)


def test_batch_posterior_grids_match_single_roi_and_accumulate_by_slot(cuda_lib):
    """Batched grids (exact arithmetic): ROI k's grid equals cRJMCMC's PGrid
    for the same chain; with grid_slot, ROIs sharing a slot add up."""
    import torch
    b, rj = _c0(6, steps=300)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    Z = int(p.Grid_Zoom)
    gs = 16 * Z * 16 * Z
    dev = {k: torch.from_numpy(v).cuda() for k, v in
           (("data", b.data), ("offsets", b.offsets), ("xsize", b.xsize), ("ysize", b.ysize))}
    dev["side_max"] = 16
    s = sampler.Sampler()

    def run(slots):
        ng = 6 if slots is None else int(max(slots)) + 1
        outs = {"status": torch.zeros(6, dtype=torch.int32, device="cuda"),
                "pgrid": torch.zeros(ng * gs, dtype=torch.float32, device="cuda"),
                "pback": torch.zeros(ng * gs, dtype=torch.float32, device="cuda"), "grid_stride": gs}
        if slots is not None:
            outs["grid_slot"] = torch.tensor(slots, dtype=torch.int32, device="cuda")
        s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=13, arith="exact", outs=outs,
                     bg0=bg0)
        torch.cuda.synchronize()
        assert (outs["status"] == 0).all()
        return outs["pgrid"].cpu().numpy().reshape(ng, 16 * Z, 16 * Z)  # [g][x][y]

    own = run(None)
    for k in (0, 3):
        one = sampler.crjmcmc_raw(b.roi(k), p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons,
                                  e0=([], [], [], bg0), rng=(13, k, 0), record=False)
        np.testing.assert_array_equal(own[k].T, one["pgrid"])
    assert own.sum() > 0
    shared = run([0, 0, 1, 1, 2, 2])
    for g in range(3):
        np.testing.assert_array_equal(shared[g], own[2 * g] + own[2 * g + 1])


def test_fast_and_exact_posterior_counts_agree_on_uneven_rois(cuda_lib):
    """Fast and exact arithmetic sample the same posterior: on 2000 ROIs of
    sides 8..24 the posterior-mean emitter count (second half of each
    chain's count trace), averaged over the ROIs and two seeds, agrees
    within 0.03.  (The MAP count is a noisier statistic here: independent
    chains on ROIs with a multimodal count move its mean by ~0.04; a wrong
    stencil in fast mode once shifted it by 0.13.)"""
    b = synth.roi_batch_uneven(2000, seed=17)
    rj = rjstruct.uneven_rjstruct()
    rj.N_Burnin = rj.N_Trials = 2000
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    s = sampler.Sampler()

    def post_mean(arith, seed):
        r = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=seed, arith=arith, bg0=bg0,
                       trace_len=4000)
        assert (r["status"] == 0).all()
        m = [r["n_trace"][k, e // 2:e].mean() for k, e in enumerate(r["n_entries"])]
        return float(np.mean(m)), float(r["map_n"].mean())

    ex = [post_mean("exact", sd) for sd in (9, 10)]
    fa = [post_mean("fast", sd) for sd in (9, 10)]
    print("posterior-mean N exact", ex, "fast", fa)
    pe, pf = np.mean([e[0] for e in ex]), np.mean([f[0] for f in fa])
    assert abs(pf - pe) < 0.03, (pf, pe)
    assert abs(np.mean([e[1] for e in ex]) - np.mean([f[1] for f in fa])) < 0.1


def test_autotune_picks_a_shape_per_class_and_keeps_results(cuda_lib):
    """The autotuner times every CTA shape per size class; batches after it
    use the tuned shapes and give the same chains as before."""
    import torch
    b = synth.roi_batch_uneven(3000, seed=23)
    rj = rjstruct.uneven_rjstruct()
    rj.N_Burnin = rj.N_Trials = 300
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    dev = {"data": torch.from_numpy(b.data).cuda(), "offsets": torch.from_numpy(b.offsets).cuda(),
           "xsize": torch.from_numpy(b.xsize).cuda(), "ysize": torch.from_numpy(b.ysize).cuda(),
           "psf_sigma": torch.from_numpy(b.sigma).cuda(), "side_max": 24}
    s = sampler.Sampler()

    def run():
        outs = {k: torch.zeros(3000, dtype=torch.int32, device="cuda") for k in ("map_n", "final_n", "status")}
        outs["final_state"] = torch.zeros((3000, 4 + 4 * 32), dtype=torch.float32, device="cuda")
        s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=3, arith="fast", outs=outs, bg0=bg0)
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in outs.items()}

    before = run()
    tuned = s.autotune(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, arith="fast", jumps=100,
                       sample=1000, bg0=bg0)
    print("chains per CTA by size class:", tuned)
    assert [t > 0 for t in tuned[:5]] == [True] * 5 and tuned[5:] == [0, 0]
    assert all(t in (1, 2, 4, 8) for t in tuned[:5])
    shapes, budget = s.tuned_shapes("fast")
    assert shapes == tuned and all(b in (2, 3) for b in budget[:5]) and budget[5:] == [0, 0]
    after = run()
    for k in before:
        np.testing.assert_array_equal(before[k], after[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["fast", "exact"])
def test_captured_batch_graph_replays_eager_results_on_new_data(cuda_lib, arith):
    """A batch captured as a CUDA graph gives the eager call's results, and
    replayed after new pixels are written into the same buffers it gives the
    eager results of the new pixels."""
    import torch
    n = 1500
    rj = rjstruct.uneven_rjstruct()
    rj.N_Burnin = rj.N_Trials = 200
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    b1 = synth.roi_batch_uneven(n, seed=41)
    rng = np.random.default_rng(5)
    data2 = (b1.data + rng.poisson(3.0, size=b1.data.shape)).astype(np.float32)
    dev = {"data": torch.from_numpy(b1.data).cuda(), "offsets": torch.from_numpy(b1.offsets).cuda(),
           "xsize": torch.from_numpy(b1.xsize).cuda(), "ysize": torch.from_numpy(b1.ysize).cuda(),
           "psf_sigma": torch.from_numpy(b1.sigma).cuda(), "side_max": 24}
    s = sampler.Sampler()

    def new_outs():
        o = {k: torch.zeros(n, dtype=torch.int32, device="cuda") for k in ("map_n", "final_n", "status", "n_entries")}
        o["final_state"] = torch.zeros((n, 4 + 4 * 32), dtype=torch.float32, device="cuda")
        o["counters"] = torch.zeros((n, 30), dtype=torch.int32, device="cuda")
        return o

    def eager():
        o = new_outs()
        s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=9, arith=arith, outs=o, bg0=bg0)
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in o.items()}

    ref1 = eager()
    outs = new_outs()
    g = s.capture(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=9, arith=arith, outs=outs, bg0=bg0)
    for k in outs:
        outs[k].zero_()
    st = torch.cuda.Stream()
    g.launch(st.cuda_stream)
    st.synchronize()
    for k, v in ref1.items():
        np.testing.assert_array_equal(outs[k].cpu().numpy(), v, err_msg=k)
    dev["data"].copy_(torch.from_numpy(data2))
    ref2 = eager()
    assert not np.array_equal(ref2["final_state"], ref1["final_state"])
    g.launch(st.cuda_stream)
    st.synchronize()
    for k, v in ref2.items():
        np.testing.assert_array_equal(outs[k].cpu().numpy(), v, err_msg=k)
    g.close()


@pytest.mark.parametrize("k", [0, 3])
def test_exact_chain_all_moves_background_emitters_and_scmos(cuda_lib, oracle_port, k):
    """Settings the plain workload does not reach, bit for bit against the
    oracle: all 8 move types (gSplit, gMerge, backFore on), IsBackg = 1 with
    a background-emitter prior, an sCMOS correction map, drift, a start
    state and a nonzero stream offset."""
    b, rj = _c0(6, steps=1000, seed=5)
    rj.P_Burnin = [0.3, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1]
    rj.P_Trials = [0.4, 0.0, 0.0, 0.05, 0.05, 0.15, 0.15, 0.2]
    rj.IsBackg = 1
    p = rjstruct.mcmc_params(rj, drift_x=0.3, drift_y=-0.2)
    grid = np.arange(0, 12001, 10.0)
    back = synth.lognormal_pdf(grid, 200.0, 0.5).astype(np.float32)
    rng = np.random.default_rng(k)
    roi = b.roi(k)
    scmos = rng.uniform(0.0, 3.0, roi.shape).astype(np.float32)
    e0 = (b.true_i[k].astype(np.float32), b.true_x[k].astype(np.float32), b.true_y[k].astype(np.float32), 8.0)
    args = (p, rj.P_Offset, rj.P_EmPhotons, back)
    ref = oracle_port.run_chain("port", roi, *args, e0=e0, rng=(3, 500 + k, 11), scmos=scmos)
    got = sampler.crjmcmc_raw(roi, *args, e0=e0, rng=(3, 500 + k, 11), scmos=scmos, arith="exact")
    assert ref["counters"]["N_birthBg"] > 1 or ref["counters"]["N_jumpBg"] > 1   # background emitters appear
    assert_same_chain(got, ref)


def test_fast_sampler_matches_the_reference_posterior_ks(cuda_lib, oracle_port):
    """With its own RNG and move-synchronous CTAs, the fast sampler draws
    from the posterior of the reference algorithm: on one ROI, the final
    states of 384 independent GPU chains and of 192 oracle chains (the C
    restatement, bit-identical to the reference build; independent streams)
    agree in the emitter count (total variation) and in the emitters' X and
    Y positions (two-sample Kolmogorov-Smirnov)."""
    import concurrent.futures as cf
    from scipy.stats import ks_2samp
    b0, rj = _c0(8, steps=2000, seed=6)
    k = int(np.argsort(b0.true_n)[len(b0.true_n) // 2])
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    roi = b0.roi(k)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)

    def oracle_final(c):
        r = oracle_port.run_chain("port", roi, *args, e0=([], [], [], bg0), rng=(77, 10000 + c, 0))
        ch = r["chain"]
        n, I, X, Y, S = sampler._emitters_of(ch, len(ch["N"]) - 1)
        keep = (S == 1) if int(ch["N"][-1]) > 0 else np.zeros(0, bool)
        return int(ch["N"][-1]), X[keep], Y[keep]

    with cf.ThreadPoolExecutor(16) as ex:
        ora = list(ex.map(oracle_final, range(192)))
    copies = 384
    b = synth._pack([roi] * copies, [b0.sigma[k]] * copies, [b0.bg[k]] * copies, [b0.true_n[k]] * copies,
                    [b0.true_x[k]] * copies, [b0.true_y[k]] * copies, [b0.true_i[k]] * copies)
    s = sampler.Sampler()
    got = s.run_host(b, *args, seed=41, arith="fast", bg0=bg0)
    assert (got["status"] == 0).all()
    fs, fn = got["final_state"], got["final_n"]
    nmax = (fs.shape[1] - 4) // 4
    gx = np.concatenate([fs[i, 4 + nmax:4 + nmax + fn[i]][fs[i, 4 + 3 * nmax:4 + 3 * nmax + fn[i]] == 1]
                         for i in range(copies)])
    gy = np.concatenate([fs[i, 4 + 2 * nmax:4 + 2 * nmax + fn[i]][fs[i, 4 + 3 * nmax:4 + 3 * nmax + fn[i]] == 1]
                         for i in range(copies)])
    on = np.array([o[0] for o in ora])
    ox = np.concatenate([o[1] for o in ora])
    oy = np.concatenate([o[2] for o in ora])
    K = 12
    hg = np.bincount(np.minimum(fn, K - 1), minlength=K) / copies
    ho = np.bincount(np.minimum(on, K - 1), minlength=K) / len(on)
    tv = 0.5 * np.abs(hg - ho).sum()
    px = ks_2samp(gx, ox).pvalue
    py = ks_2samp(gy, oy).pvalue
    print(f"ROI {k} (true N {b0.true_n[k]}): count TV {tv:.3f}; KS p-values X {px:.3f}, Y {py:.3f}; "
          f"mean N gpu {fn.mean():.2f} oracle {on.mean():.2f}")
    assert tv < 0.12
    assert px > 0.001 and py > 0.001
