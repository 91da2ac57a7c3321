"""The sampled-PSF producers (findPSF.m, findPSF_SMA.m) and per-ROI PSF
slots of the batched sampler.

findPSF's FFT shift-and-average and findPSF_SMA's spot selection run on the
host over the GPU front end (findROI, gaussMLE 'Sigma').  MATLAB and the
absent SMA_Core are not here to pin them against, so these tests check the
properties the reference's construction implies on ideal and on noisy
spots: unit-sum planes, sub-position planes a quarter pixel apart, the
spot width, the Gaussian fallback, and that the sampler reads the PSF a
ROI's slot names."""
import numpy as np
import pytest
from scipy.special import erf

from bamf_gb300 import psf as psfmod, rjstruct, sampler, synth

pytestmark = pytest.mark.gpu


def _spots(n, sigma=1.3, box=8, photons=2000.0, bg=0.0, seed=0, noise=False):
    rng = np.random.default_rng(seed)
    X = (box - 1) / 2 + rng.uniform(-0.7, 0.7, n)     # gaussMLE coordinates: pixel centres at integers
    Y = (box - 1) / 2 + rng.uniform(-0.7, 0.7, n)
    i = np.arange(box)

    def integ(c):
        return 0.5 * (erf((i[:, None] - c[None, :] + 0.5) / (np.sqrt(2) * sigma))
                      - erf((i[:, None] - c[None, :] - 0.5) / (np.sqrt(2) * sigma)))

    lam = photons * integ(Y)[:, None, :] * integ(X)[None, :, :] + bg
    return (rng.poisson(lam) if noise else lam).astype(np.float32)


def _centroids(P):
    idx = np.arange(P.shape[0]) + 0.5
    c = np.zeros((4, 4, 2))
    w = np.zeros((4, 4))
    for jj in range(4):
        for ii in range(4):
            pl = P[:, :, jj, ii].astype(np.float64)
            c[jj, ii] = (pl.sum(1) * idx).sum(), (pl.sum(0) * idx).sum()
            w[jj, ii] = np.sqrt((pl.sum(0) * (idx - c[jj, ii, 1]) ** 2).sum())
    return c, w


@pytest.mark.parametrize("noise", [False, True])
def test_find_psf_planes(cuda_lib, noise):
    """Ideal and Poisson spots of sigma 1.3: 64 x 64 x 4 x 4, every plane
    sums to 1, sub-position planes step a quarter pixel in their axis, the
    spot is 1.15-1.35 px wide, and plane (0, 0) is centred at 32.5 (pixel
    centres at i + 0.5): half a pixel past the c0 = 32 NumModel assumes,
    the geometry of the reference's transforms for an 8-pixel box with
    gaussMLE's coordinates (pixel edges at integers)."""
    stack = _spots(300, noise=noise, bg=5.0 if noise else 0.0)
    P = psfmod.find_psf(stack, 1.0, 5.0 if noise else 0.0, 1.3, 8)
    assert P.shape == (64, 64, 4, 4) and P.dtype == np.float32
    np.testing.assert_allclose(P.sum(axis=(0, 1)), 1.0, atol=1e-5)
    c, w = _centroids(P)
    tol = 0.03 if not noise else 0.06
    for jj in range(4):
        for ii in range(4):
            assert abs(c[jj, ii, 0] - (32.5 + jj / 4)) < tol, (jj, ii, c[jj, ii])
            assert abs(c[jj, ii, 1] - (32.5 + ii / 4)) < tol, (jj, ii, c[jj, ii])
    assert 1.15 < w.min() and w.max() < 1.35, w
    with pytest.raises(ValueError):
        psfmod.find_psf(stack[:7, :7], 1.0, 0.0, 1.3, 7)


def test_find_psf_sma_per_position_and_fallback(cuda_lib):
    """Sparse frames with bright isolated emitters give each sub-region
    position its own PSF from the spots found there; positions with fewer
    than 30 usable spots fall back to the Gaussian spot of sigma PSF_Sigma."""
    from bamf_gb300 import tiles
    frames, _, _ = synth.frames_dense(120, size=40, seed=4, density=(0.8, 1.2), median_i=2500.0, log_sd=0.2,
                                      bg=(5.0, 10.0))
    ROI_Data, S, _ = tiles.makeSubRegions(frames, 10, 3)
    stacks = psfmod.tile_stacks(ROI_Data, S)
    assert len(stacks) == S["Xsub"] * S["Ysub"]
    psfs = psfmod.find_psf_sma(stacks, 1.3, 2500.0, 8)
    assert len(psfs) == len(stacks)
    for P in psfs:
        assert P.shape == (64, 64, 4, 4)
        np.testing.assert_allclose(P.sum(axis=(0, 1)), 1.0, atol=1e-5)
        c, w = _centroids(P)
        assert np.all(np.abs(c[..., 0] - (32.5 + np.arange(4)[:, None] / 4)) < 0.15)
        assert 1.0 < w.min() and w.max() < 1.5
    empty = [np.random.default_rng(1).poisson(8.0, (16, 16, 5)).astype(np.float32)]
    fb = psfmod.find_psf_sma(empty, 1.3, 2500.0, 8)[0]
    g = np.arange(0.5, 8, 1.0)
    xg, yg = np.meshgrid(g, g)
    spot = 2500.0 * psfmod._normpdf(xg, 4, 1.3) * psfmod._normpdf(yg, 4, 1.3)
    ref = psfmod.find_psf(np.repeat(spot[:, :, None], 50, axis=2), 1.0, 0.0, 1.3, 8)
    np.testing.assert_array_equal(fb, ref)


def test_batch_reads_each_rois_psf_slot(cuda_lib, oracle_port):
    """Two PSFs (sigma 1.3 and 1.0) and alternating slots: every ROI's exact
    chain is the oracle chain with its own PSF; a slot outside [0, n_psf)
    fails that ROI alone."""
    from bamf_gb300.abi import COUNTER_NAMES
    n = 12
    b = synth.roi_batch_c0(n, seed=2)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = 400
    p = rjstruct.mcmc_params(rj)
    psfs = np.stack([psfmod.gaussian_sampled_psf(1.3, 48), psfmod.gaussian_sampled_psf(1.0, 48)])
    for k, v in enumerate(psfs.shape[1:]):
        p.PSFsize[k] = v
    bg0 = rjstruct.initial_bg(rj)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    slot = (np.arange(n) % 2).astype(np.int32)
    s = sampler.Sampler()
    got = s.run_host(b, *args, seed=9, arith="exact", bg0=bg0, sampled_psf=psfs, psf_slot=slot)
    assert (got["status"] == 0).all()
    for k in range(n):
        ref = oracle_port.run_chain("port", b.roi(k), *args, e0=([], [], [], bg0), rng=(9, k, 0),
                                    sampled_psf=psfs[slot[k]])
        assert got["final_n"][k] == ref["chain"]["N"][-1], k
        assert [int(v) for v in got["counters"][k]] == [ref["counters"][m] for m in COUNTER_NAMES], k
    bad = slot.copy()
    bad[3] = 2
    got2 = s.run_host(b, *args, seed=9, arith="fast", bg0=bg0, sampled_psf=psfs, psf_slot=bad)
    assert got2["status"][3] != 0
    assert (np.delete(got2["status"], 3) == 0).all()
