"""GPU parity of the sampled-PSF likelihood model (OptModel 1, NumModel of
source/c/LibRJMCMC.cpp:67-170) against the CPU oracle, which the
reference's own build pins (tests/golden/rjmcmc_ref_numpsf.npz).

Exact arithmetic reproduces the oracle chain bit for bit, including reads
clamped at the end of a PSF array too small for the ROI; fast arithmetic
agrees in distribution; with the Gaussian PSF sampled at 4 x 4 sub-pixel
positions the sampled model finds the emitter counts the Gaussian model
finds."""
import numpy as np
import pytest

from bamf_gb300 import psf as psfmod, rjstruct, sampler, synth

from test_sampler_gpu import assert_same_chain

pytestmark = pytest.mark.gpu


def _setup(n_rois, steps, psf, seed=0):
    b = synth.roi_batch_c0(n_rois, seed=seed)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = steps
    p = rjstruct.mcmc_params(rj)
    for k, v in enumerate(psf.shape):
        p.PSFsize[k] = v
    return b, rj, p, rjstruct.initial_bg(rj)


GAUSS = psfmod.gaussian_sampled_psf(1.3)
SMALL = (np.random.default_rng(1).random((10, 10, 2, 2)) * 0.05).astype(np.float32)


@pytest.mark.parametrize("case,k", [("gauss64", 0), ("gauss64", 3), ("small10", 1)])
def test_exact_chain_sampled_psf_matches_oracle(cuda_lib, oracle_port, case, k):
    psf = GAUSS if case == "gauss64" else SMALL
    b, rj, p, bg0 = _setup(4, 1200, psf)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    ref = oracle_port.run_chain("port", b.roi(k), *args, e0=([], [], [], bg0), rng=(13, k, 0), sampled_psf=psf)
    got = sampler.crjmcmc_raw(b.roi(k), *args, e0=([], [], [], bg0), rng=(13, k, 0), arith="exact",
                              sampled_psf=psf)
    assert_same_chain(got, ref)


def test_exact_chain_sampled_psf_start_state_all_moves(cuda_lib, oracle_port):
    """All 8 move types, background emitters (IsBackg = 1, a background
    prior), an sCMOS map, drift, a start state and a nonzero stream offset."""
    b, rj, p, _ = _setup(4, 800, GAUSS, seed=3)
    rj.P_Burnin = [0.3, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1]
    rj.P_Trials = [0.4, 0.0, 0.0, 0.05, 0.05, 0.15, 0.15, 0.2]
    rj.IsBackg = 1
    p = rjstruct.mcmc_params(rj, drift_x=0.3, drift_y=-0.2)
    for i, v in enumerate(GAUSS.shape):
        p.PSFsize[i] = v
    k = 2
    back = synth.lognormal_pdf(np.arange(0, 12001, 10.0), 200.0, 0.5).astype(np.float32)
    scmos = np.random.default_rng(4).uniform(0.0, 3.0, b.roi(k).shape).astype(np.float32)
    e0 = (b.true_i[k].astype(np.float32), b.true_x[k].astype(np.float32), b.true_y[k].astype(np.float32), 8.0)
    args = (p, rj.P_Offset, rj.P_EmPhotons, back)
    ref = oracle_port.run_chain("port", b.roi(k), *args, e0=e0, rng=(5, 77, 21), sampled_psf=GAUSS, scmos=scmos)
    got = sampler.crjmcmc_raw(b.roi(k), *args, e0=e0, rng=(5, 77, 21), arith="exact", sampled_psf=GAUSS,
                              scmos=scmos)
    assert_same_chain(got, ref)


def test_exact_batch_sampled_psf_matches_oracle(cuda_lib, oracle_port):
    """Batch path (host and device entry points): final emitter count and
    the 30 counters of every ROI against single oracle chains."""
    import torch
    n = 24
    b, rj, p, bg0 = _setup(n, 600, GAUSS)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    s = sampler.Sampler()
    got = s.run_host(b, *args, seed=17, arith="exact", bg0=bg0, sampled_psf=GAUSS)
    assert (got["status"] == 0).all()
    from bamf_gb300.abi import COUNTER_NAMES
    for k in range(n):
        ref = oracle_port.run_chain("port", b.roi(k), *args, e0=([], [], [], bg0), rng=(17, k, 0),
                                    sampled_psf=GAUSS)
        assert got["final_n"][k] == ref["chain"]["N"][-1], k
        assert [int(v) for v in got["counters"][k]] == [ref["counters"][m] for m in COUNTER_NAMES], k
    dev = {"data": torch.from_numpy(b.data).cuda(), "offsets": torch.from_numpy(b.offsets).cuda(),
           "xsize": torch.from_numpy(b.xsize).cuda(), "ysize": torch.from_numpy(b.ysize).cuda(),
           "psf_sigma": torch.from_numpy(b.sigma).cuda(), "side_max": int(max(b.xsize.max(), b.ysize.max())),
           "sampled_psf": torch.from_numpy(np.ascontiguousarray(GAUSS.ravel(order="F"))).cuda()}
    outs = {k: torch.zeros(n, dtype=torch.int32, device="cuda") for k in ("final_n", "status", "map_n")}
    outs["counters"] = torch.zeros((n, 30), dtype=torch.int32, device="cuda")
    s.run_device(dev, *args, seed=17, arith="exact", outs=outs, bg0=bg0)
    torch.cuda.synchronize()
    for k in ("final_n", "counters", "map_n"):
        np.testing.assert_array_equal(outs[k].cpu().numpy(), got[k], err_msg=k)


def test_fast_sampled_psf_agrees_with_exact_and_with_gaussian_model(cuda_lib):
    """Fast arithmetic with the sampled PSF: the posterior emitter counts
    agree with exact arithmetic, and the 4 x 4-sampled Gaussian PSF gives
    the counts the Gaussian model gives."""
    n = 512
    b, rj, p, bg0 = _setup(n, 1500, GAUSS)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    s = sampler.Sampler()
    ex = s.run_host(b, *args, seed=3, arith="exact", bg0=bg0, sampled_psf=GAUSS)
    fa = s.run_host(b, *args, seed=3, arith="fast", bg0=bg0, sampled_psf=GAUSS)
    ga = s.run_host(b, *args, seed=3, arith="fast", bg0=bg0)
    for r in (ex, fa, ga):
        assert (r["status"] == 0).all() and (r["overflow"] == 0).all()
    print("map_n mean: exact %.3f fast %.3f gaussian %.3f truth %.3f" % (
        ex["map_n"].mean(), fa["map_n"].mean(), ga["map_n"].mean(), b.true_n.mean()))
    assert np.mean(fa["map_n"] == ex["map_n"]) > 0.6
    assert abs(fa["map_n"].mean() - ex["map_n"].mean()) < 0.25
    assert np.mean(fa["map_n"] == ga["map_n"]) > 0.6
    assert abs(fa["map_n"].mean() - ga["map_n"].mean()) < 0.25


def test_sampled_psf_arguments_are_checked(cuda_lib):
    b, rj, p, bg0 = _setup(4, 10, GAUSS)
    s = sampler.Sampler()
    bad = rjstruct.mcmc_params(rj)
    bad.PSFsize[2] = 0
    with pytest.raises(Exception):
        s.run_host(b, bad, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1, sampled_psf=np.zeros((64, 64, 0, 4)))
    with pytest.raises(ValueError):
        s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1, sampled_psf=SMALL)
