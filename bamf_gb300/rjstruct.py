"""RJStruct defaults and the per-call MCMC struct, as the reference builds them.

RJStruct mirrors genRJStruct.m:43-63; mcmc_params() is rjmcmc.m:43-78 (the
struct handed to cRJMCMC) and refine_params() is mcmc.m:103-138 (the
fixed-N refinement call with P = [1 0 0 0 0 0 0 0] and IsBackg = 0).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import synth
from .abi import McmcParams


@dataclass
class RJStruct:
    SRZoom: int = 20
    P_EmPhotons: np.ndarray | None = None
    P_BgEmPhotons: np.ndarray | None = None
    P_Offset: np.ndarray | None = None
    PSF_Sigma: float = 1.3
    N_Trials: int = 2000
    N_Burnin: int = 3000
    N_TrialsMCMC: int = 1000
    N_BurninMCMC: int = 1000
    P_Burnin: list = field(default_factory=lambda: [0.3, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1])
    P_Trials: list = field(default_factory=lambda: [0.4, 0, 0, 0.05, 0.05, 0.15, 0.15, 0.2])
    P_dP: float = 10.0
    Rho: float = 0.01
    MinPhoton: float = 0.0
    XstdFg: float = 0.1
    IstdFg: float = 10.0
    BGstd: float = 1.0
    IsBackg: int = 1
    BgPriorRange: float = 12.0


def _f32(x) -> float:
    return float(np.float32(x))


def mcmc_params(rj: RJStruct, drift_x: float = 0.0, drift_y: float = 0.0) -> McmcParams:
    """The `MCMC` struct of rjmcmc.m:49-78 (all single/int32 as MATLAB casts)."""
    p = McmcParams()
    p.PSFsigma = _f32(rj.PSF_Sigma)
    p.Grid_Zoom = int(rj.SRZoom)
    p.N_Trials = int(rj.N_Trials)
    p.N_Burnin = int(rj.N_Burnin)
    p.I_stdFg = _f32(rj.IstdFg)
    p.I_stdBg = _f32(rj.IstdFg / 2)
    p.X_stdFg = _f32(rj.XstdFg)
    p.X_stdBg = _f32(rj.XstdFg / 2)
    for k in range(8):
        p.P_Burnin[k] = _f32(rj.P_Burnin[k])
        p.P_Trials[k] = _f32(rj.P_Trials[k])
    p.Split_std = _f32(0.5)
    p.Bnd_out = _f32(2)
    p.Icutoff = _f32(rj.MinPhoton)
    p.Rho = _f32(rj.Rho)
    p.BG_std = _f32(rj.BGstd)
    p.ABBG_std = _f32(0.02)
    p.DX = _f32(rj.P_dP)
    p.DriftX = _f32(drift_x)
    p.DriftY = _f32(drift_y)
    p.IsBackg = int(rj.IsBackg)
    for k, v in enumerate((10, 10, 2, 2)):
        p.PSFsize[k] = v
    return p


def refine_params(rj: RJStruct, drift_x: float = 0.0, drift_y: float = 0.0) -> McmcParams:
    """The fixed-N refinement struct of mcmc.m:103-138."""
    p = mcmc_params(rj, drift_x, drift_y)
    p.N_Trials = int(rj.N_TrialsMCMC)
    p.N_Burnin = int(rj.N_BurninMCMC)
    p.I_stdBg = _f32(rj.IstdFg / 1.5)
    p.X_stdBg = _f32(rj.XstdFg / 1.5)
    for k in range(8):
        p.P_Burnin[k] = 1.0 if k == 0 else 0.0
        p.P_Trials[k] = 1.0 if k == 0 else 0.0
    p.IsBackg = 0
    return p


def initial_bg(rj: RJStruct) -> float:
    """E_active.BG of rjmcmc.m:47: the grid position of the offset-prior max."""
    po = np.asarray(rj.P_Offset)
    return _f32(rj.P_dP * int(np.flatnonzero(po == po.max())[0]))


def c0_rjstruct(side: int = 16) -> RJStruct:
    """Sampler settings of the plain-RJMCMC workload (200 ROIs 16x16):
    move/bg/birth/death/split/merge 0.4/0.1/0.15/0.15/0.1/0.1 mapped onto the
    8-slot vector as P = [0.5, 0.1, 0.1, 0.15, 0.15, 0, 0, 0] with the
    background moves being the 25% sub-branch of `jump`; Rho = 3/256
    (MeanN = 3 on 16x16); signal prior = the generator's log-normal pdf on
    the grid 0:10:12000; offset prior = Gamma(shape 20, scale 0.5) (mean 10)
    on the same grid; no background-emitter prior (IsBackg = 0)."""
    grid = np.arange(0, 12001, 10, dtype=np.float64)
    P = [0.5, 0.1, 0.1, 0.15, 0.15, 0.0, 0.0, 0.0]
    return RJStruct(
        SRZoom=20,
        P_EmPhotons=synth.lognormal_pdf(grid, 1000.0, 0.3).astype(np.float32),
        P_BgEmPhotons=np.zeros(grid.shape, np.float32),
        P_Offset=synth.gamma_pdf(grid, 20.0, 0.5).astype(np.float32),
        PSF_Sigma=1.3, N_Trials=3000, N_Burnin=3000, P_Burnin=P, P_Trials=P,
        P_dP=10.0, Rho=3.0 / (side * side), MinPhoton=0.0, XstdFg=0.1, IstdFg=10.0,
        BGstd=1.0, IsBackg=0)


def uneven_rjstruct() -> RJStruct:
    """Sampler settings of the batched uneven workload (ROI sides
    {8,12,16,20,24}, N ~ Poisson(U[0,12]), sigma ~ U[1.1,1.5], I ~
    LogN(ln 1000, 0.4), background ~ U[5,50]): the same move mapping and
    jump counts as c0_rjstruct; Rho = 6/288 (the mean emitter count over the
    mean ROI area); signal prior = the generator's log-normal pdf; offset
    prior = the Gamma with the mean and variance of U[5,50] (shape 4.48,
    scale 6.14), as findPriors.m:66-67 fits one to measured backgrounds."""
    grid = np.arange(0, 12001, 10, dtype=np.float64)
    rj = c0_rjstruct()
    rj.P_EmPhotons = synth.lognormal_pdf(grid, 1000.0, 0.4).astype(np.float32)
    mean, var = 27.5, 45.0 ** 2 / 12.0
    rj.P_Offset = synth.gamma_pdf(grid, mean * mean / var, var / mean).astype(np.float32)
    rj.Rho = 6.0 / 288.0
    return rj
