"""The @RJ object's analyzeData (RJ.m:164-256) on the GPU: camera counts in,
gain correction, priors from the data, sub-region analysis, stitched signal
and background posteriors, the MAP emitter list."""
import numpy as np
import pytest

from bamf_gb300 import pipeline, rj as rjmod, synth

pytestmark = pytest.mark.gpu


def test_rj_analyze_data_localises_emitters(cuda_lib):
    pytest.importorskip("scipy")
    frames, truth, _ = synth.frames_dense(3, size=64, seed=8, density=(1.0, 1.5), median_i=1500.0, log_sd=0.3,
                                          bg=(20.0, 40.0))
    obj = rjmod.RJ()
    obj.Data = frames * 2.0 + 100.0           # camera counts: gain 2, offset 100
    obj.Camera_Gain, obj.Camera_Offset = 2.0, 100.0
    obj.BoxSize, obj.Overlap = 10, 3
    obj.RJStruct.N_Burnin = obj.RJStruct.N_Trials = 2000
    obj.RJStruct.N_BurninMCMC = obj.RJStruct.N_TrialsMCMC = 500
    obj.RJStruct.SRZoom = 4
    obj.RJStruct.Rho = 0.012
    obj.analyzeData(proposal="reference", seed=5)
    st = pipeline.localisation_stats(obj.ClustInfo, truth)
    print(st)
    assert obj.PImage.shape == (4 * 64, 4 * 64) and obj.PBg.shape == obj.PImage.shape
    assert obj.PImage.sum() > 0
    assert st["recall"] > 0.7 and st["precision"] > 0.7 and st["rmse_px"] < 0.35
    np.testing.assert_allclose(obj.Data, frames, rtol=1e-6)   # gain-corrected in place
