"""The @RJ analysis object (@RJ/RJ.m) over this library: the properties a
user of the reference sets, and analyzeData (RJ.m:164-256):
gain correction, priors from the data (findPriors), optionally sampled PSFs
from the data (FindPSF = 1, findPSF_SMA), then the sub-region analysis on
the GPU (makeSubRegions, the batched sampler, findMap + mcmc refinement,
removeOverlapping and stitchROIs of the signal and background posteriors).

Differences from the MATLAB object: one GPU replaces the parfor over frame
blocks (UsePPToolbox is ignored); chains are not kept (KeepChain = 0 only);
the GUI, thresholding, frame connection and drift correction around the
analysis are not part of this library.
"""
from __future__ import annotations

import numpy as np

from . import pipeline, priors, psf, rjstruct, tiles


class RJ:
    def __init__(self):
        self.RJStruct = rjstruct.RJStruct()      # genRJStruct defaults
        self.Data = None                         # Y x X x frames, camera counts
        self.Camera_Gain = 11.0
        self.Camera_Offset = 100.0
        self.Camera_Var = None
        self.BoxSize = 16
        self.Overlap = 3
        self.SMAStruct = {"MeanPhotons": 800.0, "MinPValue": 0.01, "MinPhotons": 100.0}
        self.SampledPSF = []
        self.FindPSF = 0
        self.FindPriors = 1
        self.PImage = None
        self.PBg = None
        self.ClustInfo = None
        self.ROI_Data = None

    def gainCorrection(self) -> None:
        """RJ.m:161: Data = (Data - Camera_Offset) / Camera_Gain in single."""
        d = np.asarray(self.Data, np.float32)
        self.Data = ((d - np.float32(self.Camera_Offset)) / np.float32(self.Camera_Gain)).astype(np.float32)

    def analyzeData(self, proposal: str = "reference", net=None, seed: int = 1) -> "RJ":
        """RJ.m:164-256 for one GPU.  proposal: the sampler's birth proposal
        ("reference" reproduces the reference algorithm; "learned" needs the
        proposal network `net` and BoxSize + 2 Overlap = 16)."""
        if self.Data is None:
            raise ValueError("RJ.Data is empty")
        self.gainCorrection()
        if not self.RJStruct.PSF_Sigma:
            self.RJStruct.PSF_Sigma = 1.3
        if not self.RJStruct.P_dP:
            self.RJStruct.P_dP = 10.0
        if self.FindPriors:
            priors.findPriors(self.Data, self.RJStruct, self.SMAStruct, "Yes", self.RJStruct.BgPriorRange)
        elif self.RJStruct.P_EmPhotons is None or self.RJStruct.P_BgEmPhotons is None or \
                self.RJStruct.P_Offset is None:
            raise ValueError("Priors Must be given.")
        sampled = None
        if self.FindPSF == 1:
            ROI_Data, S, _ = tiles.makeSubRegions(self.Data, self.BoxSize, self.Overlap)
            self.SampledPSF = psf.find_psf_sma(psf.tile_stacks(ROI_Data, S), float(self.RJStruct.PSF_Sigma),
                                               float(self.SMAStruct["MeanPhotons"]),
                                               int(self.SMAStruct.get("BoxSize", 8)))
            sampled = np.stack(self.SampledPSF)
        out = pipeline.analyze_frames(np.asarray(self.Data, np.float32), self.RJStruct, box=self.BoxSize,
                                      overlap=self.Overlap, proposal=proposal, net=net, seed=seed,
                                      sampled_psf=sampled)
        self.PImage = out["PImage"].cpu().numpy()
        self.PBg = out["PBg"].cpu().numpy()
        self.ClustInfo = out["ClustInfo"]
        return self
