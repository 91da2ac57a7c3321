"""The frame analysis pipeline end to end on a few dense frames: priors from
the front end, sub-regions, batched sampler (uniform and learned births),
MAP + refinement, frame coordinates, stitched posterior image."""
import numpy as np
import pytest

from bamf_gb300 import pipeline, priors, rjstruct, synth

pytestmark = pytest.mark.gpu


def _rj(frames):
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = 3000
    rj.N_BurninMCMC = rj.N_TrialsMCMC = 1000
    rj.SRZoom = 4
    priors.findPriors(frames, rj, {"MeanPhotons": 800.0, "MinPValue": 0.01, "MinPhotons": 100.0}, "No")
    rj.Rho = 0.012
    return rj


@pytest.mark.parametrize("proposal", ["uniform", "learned"])
def test_pipeline_localises_dense_frames(cuda_lib, proposal):
    pytest.importorskip("scipy")
    from bamf_gb300 import learned
    frames, truth, _ = synth.frames_dense(3, size=64, seed=8, density=(1.0, 1.5), median_i=1500.0, log_sd=0.3,
                                          bg=(20.0, 40.0))
    rj = _rj(frames)
    net = None
    if proposal == "learned":
        net = learned.ProposalNet(seed=2)
        net.train(300, batch=512, lr=2e-3, data_seed=5, mean_n=0.012 * 256, i_median=1500.0, i_logsd=0.3,
                  bg=20.0, bg_max=40.0)
    out = pipeline.analyze_frames(frames, rj, box=10, overlap=3, proposal=proposal, net=net, seed=3)
    st = pipeline.localisation_stats(out["ClustInfo"], truth)
    print(proposal, st, {k: round(v, 3) for k, v in out["timing"].items()})
    assert out["n_subregions"] == 3 * 7 * 7
    assert abs(st["bias_x"]) < 0.05 and abs(st["bias_y"]) < 0.05
    assert st["recall"] > 0.75 and st["precision"] > 0.8 and st["rmse_px"] < 0.3
    img = out["PImage"].cpu().numpy()
    assert img.shape == (4 * 64, 4 * 64) and img.sum() > 0


def test_pipeline_with_sampled_psfs_from_the_data(cuda_lib):
    """FindPSF = 1 (RJ.m:196-197): findPSF_SMA's per-position PSFs from the
    frames themselves, then the pipeline with the sampled-PSF model.  The
    reference's findPSF centres its array half a pixel past NumModel's
    centre pixel in x and y (the geometry of its transforms with gaussMLE
    coordinates), so the emitters it finds sit about half a pixel up and
    left of the truth; localisation is checked after removing that offset."""
    from bamf_gb300 import psf as psfmod, tiles
    frames, truth, _ = synth.frames_dense(3, size=64, seed=8, density=(1.0, 1.5), median_i=1500.0, log_sd=0.3,
                                          bg=(20.0, 40.0))
    rj = _rj(frames)
    iso, _, _ = synth.frames_dense(60, size=64, seed=9, density=(0.3, 0.5), median_i=1500.0, log_sd=0.3,
                                   bg=(20.0, 40.0))
    ROI_Data, S, _ = tiles.makeSubRegions(iso, 10, 3)
    psfs = np.stack(psfmod.find_psf_sma(psfmod.tile_stacks(ROI_Data, S), 1.3, 1500.0, 8))
    out = pipeline.analyze_frames(frames, rj, box=10, overlap=3, proposal="uniform", seed=3, sampled_psf=psfs)
    ci = out["ClustInfo"]
    raw = pipeline.localisation_stats(ci, truth, radius=2.5)
    shifted = dict(ci)
    shifted["X"] = np.asarray(ci["X"]) - raw["bias_x"]
    shifted["Y"] = np.asarray(ci["Y"]) - raw["bias_y"]
    st = pipeline.localisation_stats(shifted, truth)
    print("sampled PSF: raw", raw, "offset-corrected", st)
    assert -0.6 < raw["bias_x"] < -0.3 and -0.6 < raw["bias_y"] < -0.3
    assert st["recall"] > 0.8 and st["precision"] > 0.85 and st["rmse_px"] < 0.35
