"""findPriors end to end: GPU FindROI + gaussMLE on synthetic frames, then
the threshold, kernel-density and gamma-fit statistics."""
import numpy as np
import pytest

from bamf_gb300 import priors, rjstruct, synth

pytestmark = pytest.mark.gpu


def test_find_priors_recovers_the_generator(cuda_lib):
    pytest.importorskip("scipy")
    stack, truth = synth.frames(60, size=128, seed=4, density=15.0, median_i=1500.0, log_sd=0.3, bg=20.0)
    rj = rjstruct.c0_rjstruct()
    sma = {"MeanPhotons": 1500.0, "MinPValue": 0.01, "MinPhotons": 100.0}
    sig, off, back, info = priors.findPriors(stack, rj, sma, "Yes", BgPriorRange=10.0)
    print(info)
    grid = np.arange(len(sig)) * rj.P_dP
    assert info["n_kept"] > 200
    mode = grid[np.argmax(sig)]
    assert abs(mode / 1500.0 - 1) < 0.25, mode
    assert abs(sig.sum() * rj.P_dP - 1) < 0.02
    assert abs(info["gamma_shape"] * info["gamma_scale"] / 20.0 - 1) < 0.15
    assert len(off) == len(sig) == len(back) and back[0] > 0
    assert rj.P_EmPhotons is sig and rj.P_Offset is off
