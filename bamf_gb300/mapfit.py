"""MAP emitter sets and fixed-count refinement of a batch (@RJ/findMap.m,
@RJ/mcmc.m, as analyzeROIs.m:150-160 chains them), on the GPU.

  pass 1  the batched sampler with a thinned state trace (pos_trace)
  map     bamf_map_kmeans_device: MAP count, k-means of the MAP-count
          states' positions, per-cluster mean / std (findMap.m)
  pass 2  for ROIs with a MAP count > 0, the jumps-only sampler
          (refine_params: mcmc.m:103-138) started from the k-means means
  refine  bamf_refine_stats_device: per-emitter mean / std over the second
          half of the refinement chain (mcmc.m:142-169)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi, rjstruct, sampler

POS_SLOTS = 32
POS_RECORD = 5 + 3 * POS_SLOTS
MAP_RECORD = 6 + 6 * POS_SLOTS
MAX_POS_LEN = 256


def _lib():
    L = abi.lib()
    if getattr(L, "_mapfit_declared", False):
        return L
    vp, i32 = C.c_void_p, C.c_int
    L.bamf_map_kmeans_device.restype = C.c_int
    L.bamf_map_kmeans_device.argtypes = [vp, i32, i32, vp, vp, i32, i32, vp, vp]
    L.bamf_refine_stats_device.restype = C.c_int
    L.bamf_refine_stats_device.argtypes = [vp, i32, i32, vp, i32, vp, vp]
    L._mapfit_declared = True
    return L


def thinning(steps: int, pos_len: int = 250) -> int:
    """Record every pos_thin-th entry so that a chain of `steps` jumps fits."""
    return max(1, -(-(steps + 1) // pos_len))


def map_kmeans(pos_trace, pos_thin: int, n_entries, map_n, max_iter: int = 100, stream=None):
    import torch
    n = int(n_entries.numel())
    out = torch.empty((n, MAP_RECORD), dtype=torch.float32, device=pos_trace.device)
    abi.check(_lib().bamf_map_kmeans_device(pos_trace.data_ptr(), int(pos_trace.shape[1]), int(pos_thin),
                                            n_entries.data_ptr(), map_n.data_ptr(), n, int(max_iter),
                                            out.data_ptr(), C.c_void_p(stream) if stream else None),
              "bamf_map_kmeans_device")
    return out


def refine_stats(pos_trace, pos_thin: int, n_entries, stream=None):
    import torch
    n = int(n_entries.numel())
    out = torch.empty((n, MAP_RECORD), dtype=torch.float32, device=pos_trace.device)
    abi.check(_lib().bamf_refine_stats_device(pos_trace.data_ptr(), int(pos_trace.shape[1]), int(pos_thin),
                                              n_entries.data_ptr(), n, out.data_ptr(),
                                              C.c_void_p(stream) if stream else None),
              "bamf_refine_stats_device")
    return out


def unpack(rec: np.ndarray) -> dict:
    """Rows of BAMF_MAP_RECORD floats -> named arrays ([n] and [n][POS_SLOTS])."""
    S = POS_SLOTS
    d = {"N": np.nan_to_num(rec[:, 0]).astype(np.int64), "records": np.nan_to_num(rec[:, 1]).astype(np.int64),
         "Bg": rec[:, 2],
         "Bg_SE": rec[:, 3], "ABg": rec[:, 4], "BBg": rec[:, 5]}
    for k, name in enumerate(("X", "Y", "I", "X_SE", "Y_SE", "I_SE")):
        d[name] = rec[:, 6 + k * S:6 + (k + 1) * S]
    return d


def _set_psf_size(p, shape):
    if shape is not None:
        for k, v in enumerate(shape):
            p.PSFsize[k] = int(v)
    return p


def _run(s, dev, params, rj, seed, arith, proposal, pos_len, bg0, extra=None):
    import torch
    n = int(dev["xsize"].numel())
    steps = int(params.N_Burnin) + int(params.N_Trials)
    thin = thinning(steps, pos_len)
    outs = {k: torch.zeros(n, dtype=torch.int32, device="cuda")
            for k in ("map_n", "final_n", "status", "n_entries")}
    outs["pos_trace"] = torch.zeros((n, pos_len, POS_RECORD), dtype=torch.float32, device="cuda")
    outs["pos_thin"] = thin
    if extra:
        outs.update(extra)
    s.run_device(dev, params, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=seed, arith=arith, outs=outs,
                 bg0=bg0, proposal=proposal)
    return outs, thin


def analyze(dev: dict, rj, seed: int = 1, arith: str = "fast", proposal: str = "reference", pos_len: int = 250,
            refine: bool = True, s=None, grids: dict | None = None, sampled_psf=None, psf_slot=None) -> dict:
    """findMap + mcmc for every ROI of a device batch (sampler.run_device
    layout).  Returns numpy dicts 'map' (findMap SMD per ROI) and 'refined'
    (mcmc FoundMAP per ROI; NaN rows where the MAP count is 0), plus the
    pass-1 map_n / n_entries.  sampled_psf (one 4-D PSF or a stack of them,
    with psf_slot [n] torch int32 naming each ROI's) selects the sampled-PSF
    model for both passes, as analyzeROIs.m:142-162 does."""
    import torch
    s = s or sampler.Sampler()
    psf_shape = None
    if sampled_psf is not None:
        a = np.asarray(sampled_psf, np.float32)
        psf_shape = a.shape[-4:]
        tmp = rjstruct.mcmc_params(rj)
        _set_psf_size(tmp, psf_shape)
        flat, npsf = sampler.pack_psfs(a, tmp)
        dev = dict(dev)
        dev["sampled_psf"] = torch.from_numpy(flat).cuda()
        dev["n_psf"] = npsf
        if psf_slot is not None:
            dev["psf_slot"] = psf_slot
    p1 = _set_psf_size(rjstruct.mcmc_params(rj), psf_shape)
    bg0 = rjstruct.initial_bg(rj)
    outs, thin = _run(s, dev, p1, rj, seed, arith, proposal, pos_len, bg0, extra=grids)
    km = map_kmeans(outs["pos_trace"], thin, outs["n_entries"], outs["map_n"])
    res = {"map_n": outs["map_n"].cpu().numpy(), "n_entries": outs["n_entries"].cpu().numpy(),
           "status": outs["status"].cpu().numpy(), "map": unpack(km.cpu().numpy())}
    n = int(dev["xsize"].numel())
    refined = np.full((n, MAP_RECORD), np.nan, np.float32)
    if refine:
        K = km[:, 0].to(torch.int32)
        idx = torch.nonzero(K > 0).flatten()
        if idx.numel():
            sub = {k: dev[k].index_select(0, idx) for k in ("offsets", "xsize", "ysize") if k in dev}
            sub["data"] = dev["data"]
            if dev.get("psf_sigma") is not None:
                sub["psf_sigma"] = dev["psf_sigma"].index_select(0, idx)
            sub["side_max"] = dev.get("side_max", 0)
            if dev.get("sampled_psf") is not None:
                sub["sampled_psf"], sub["n_psf"] = dev["sampled_psf"], dev["n_psf"]
                if dev.get("psf_slot") is not None:
                    sub["psf_slot"] = dev["psf_slot"].index_select(0, idx)
            m = int(idx.numel())
            kk = K.index_select(0, idx)
            ixy = torch.zeros((m, 3, 32), dtype=torch.float32, device="cuda")
            S = POS_SLOTS
            sel = km.index_select(0, idx)
            ixy[:, 0, :S] = torch.nan_to_num(sel[:, 6 + 2 * S:6 + 3 * S])   # I
            ixy[:, 1, :S] = torch.nan_to_num(sel[:, 6:6 + S])               # X
            ixy[:, 2, :S] = torch.nan_to_num(sel[:, 6 + S:6 + 2 * S])       # Y
            sub["init_n"] = kk.contiguous()
            sub["init_ixy"] = ixy
            sub["init_bg"] = sel[:, 2].contiguous()
            p2 = _set_psf_size(rjstruct.refine_params(rj), psf_shape)
            outs2, thin2 = _run(s, sub, p2, rj, seed + 7919, arith, "reference", pos_len, bg0)
            rs = refine_stats(outs2["pos_trace"], thin2, outs2["n_entries"])
            refined[idx.cpu().numpy()] = rs.cpu().numpy()
    res["refined"] = unpack(refined)
    return res
