"""The reference's own example (Examples/Example_SyntheticCircle.m on
Examples/Circle/CircleData.mat) through the @RJ port: the same settings
(PSF sigma 1.2 px, gain 1, offset 0, XstdFg 0.05 px, IstdFg 5 photons,
no drift), the first 400 of its 10 x 10 frames (tests/golden/
circle_example.npz, made by tests/golden/make_circle_fixture.py), and the
localisations scored against the dataset's ground truth.  The truth is in
MATLAB's 1-based pixel coordinates, the outputs 0-based: truth - 1 px is
compared (the measured offset, bias within 0.01 px)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_synthetic_circle_example_recovers_the_ground_truth(cuda_lib):
    from bamf_gb300 import pipeline, rj
    f = np.load(os.path.join(HERE, "golden", "circle_example.npz"))
    B = rj.RJ()
    B.RJStruct.PSF_Sigma = float(f["psf_sigma"])
    B.Camera_Offset = 0.0
    B.Camera_Gain = 1.0
    B.RJStruct.XstdFg = 0.05
    B.RJStruct.IstdFg = 5.0
    B.Data = f["data"]
    B.analyzeData()
    ci = B.ClustInfo
    truth = []
    for k in range(f["data"].shape[2]):
        sel = f["frame_num"] == k + 1
        truth.append((f["x"][sel] - 1.0, f["y"][sel] - 1.0, f["photons"][sel]))
    st = pipeline.localisation_stats(ci, truth, radius=1.0)
    print("circle example, 400 frames:", st)
    # measured on a GB300: precision 0.992, recall 0.750, RMSE 0.319 px,
    # bias (-0.005, 0.002) px over 1,799 true emitters (~4.5 per 10 x 10 frame)
    assert st["precision"] > 0.95
    assert st["recall"] > 0.68
    assert st["rmse_px"] < 0.37
    assert abs(st["bias_x"]) < 0.05 and abs(st["bias_y"]) < 0.05
    assert np.isfinite(B.PImage).all() and B.PImage.shape == (10 * 20, 10 * 20)
