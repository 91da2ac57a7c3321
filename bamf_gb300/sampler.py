"""Python mirror of the reference sampler interface, over libbamf_gb300.so.

  cRJMCMC(...)       the MEX function's five outputs (source/c/cRJMCMC.cpp:52-308)
  crjmcmc_raw(...)   one ROI, raw chain vectors (what the MEX marshals)
  rjmcmc(...)        @RJ/rjmcmc.m: empty start state and MCMC struct from RJStruct
  Sampler.run(...)   a whole batch of ROIs in one persistent launch

The library must be built (bamf_gb300.build.build()); there is no CPU
fallback: every call here runs the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .rjstruct import RJStruct, initial_bg, mcmc_params

ARITH = {"exact": abi.BAMF_ARITH_EXACT, "fast": abi.BAMF_ARITH_FAST}
FINAL_STRIDE = 4 + 4 * abi.BAMF_NMAX


def _declare() -> C.CDLL:
    L = abi.lib()
    if getattr(L, "_sampler_declared", False):
        return L
    pf = C.POINTER(C.c_float)
    L.bamf_crjmcmc_host.restype = C.c_int
    L.bamf_crjmcmc_host.argtypes = [
        pf, C.c_int, C.c_int, C.POINTER(abi.Emitters), C.POINTER(abi.McmcParams),
        pf, C.c_int, pf, C.c_int, pf, C.c_int, pf, C.POINTER(abi.Rng), C.c_int,
        pf, pf, C.POINTER(abi.Chain), C.POINTER(abi.Chain), C.POINTER(abi.Counters)]
    L.bamf_crjmcmc_host_model.restype = C.c_int
    L.bamf_crjmcmc_host_model.argtypes = [
        pf, C.c_int, C.c_int, C.POINTER(abi.Emitters), C.POINTER(abi.McmcParams),
        pf, C.c_int, pf, C.c_int, pf, C.c_int, pf, pf, C.c_int, C.POINTER(abi.Rng), C.c_int,
        pf, pf, C.POINTER(abi.Chain), C.POINTER(abi.Chain), C.POINTER(abi.Counters)]
    L.bamf_crjmcmc_batch_host.restype = C.c_int
    L.bamf_crjmcmc_batch_host.argtypes = [
        C.c_int, pf, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(abi.Emitters), C.POINTER(abi.McmcParams),
        C.c_void_p, pf, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int, pf, pf, C.POINTER(abi.Chain),
        C.POINTER(abi.Counters), C.c_void_p, C.c_void_p]
    L.bamf_workspace_create.restype = C.c_int
    L.bamf_workspace_create.argtypes = [C.POINTER(C.c_void_p)]
    L.bamf_workspace_destroy.argtypes = [C.c_void_p]
    L.bamf_rjmcmc_batch_device.restype = C.c_int
    L.bamf_rjmcmc_batch_device.argtypes = [C.c_void_p, C.POINTER(RoiBatch), C.POINTER(abi.McmcParams),
                                           C.POINTER(Priors), C.c_uint32, C.c_int,
                                           C.POINTER(BatchResults), C.c_void_p]
    L.bamf_rjmcmc_batch_host.restype = C.c_int
    L.bamf_rjmcmc_batch_host.argtypes = [C.c_void_p, C.POINTER(RoiBatch), C.POINTER(abi.McmcParams),
                                         C.POINTER(Priors), C.c_uint32, C.c_int,
                                         C.POINTER(BatchResults)]
    L.bamf_autotune.restype = C.c_int
    L.bamf_autotune.argtypes = [C.c_void_p, C.POINTER(RoiBatch), C.POINTER(abi.McmcParams), C.POINTER(Priors),
                                C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.bamf_autotune_result.restype = C.c_int
    L.bamf_autotune_result.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int32)]
    L.bamf_autotune_shapes.restype = C.c_int
    L.bamf_autotune_shapes.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.bamf_rjmcmc_batch_graph_create.restype = C.c_int
    L.bamf_rjmcmc_batch_graph_create.argtypes = [C.c_void_p, C.POINTER(RoiBatch), C.POINTER(abi.McmcParams),
                                                 C.POINTER(Priors), C.c_uint32, C.c_int, C.POINTER(BatchResults),
                                                 C.POINTER(C.c_void_p)]
    L.bamf_rjmcmc_batch_graph_launch.restype = C.c_int
    L.bamf_rjmcmc_batch_graph_launch.argtypes = [C.c_void_p, C.c_void_p]
    L.bamf_rjmcmc_batch_graph_destroy.argtypes = [C.c_void_p]
    L.bamf_last_error.restype = C.c_char_p
    L._sampler_declared = True
    return L


class Priors(C.Structure):
    _fields_ = [("offset_pdf", C.POINTER(C.c_float)), ("offset_len", C.c_int32),
                ("signal_pdf", C.POINTER(C.c_float)), ("signal_len", C.c_int32),
                ("back_pdf", C.POINTER(C.c_float)), ("back_len", C.c_int32)]


class RoiBatch(C.Structure):
    _fields_ = [("n_rois", C.c_int32), ("side_max", C.c_int32), ("data", C.c_void_p),
                ("offsets", C.c_void_p), ("xsize", C.c_void_p), ("ysize", C.c_void_p),
                ("psf_sigma", C.c_void_p), ("scmos", C.c_void_p), ("init_n", C.c_void_p),
                ("init_bg", C.c_void_p), ("init_ixy", C.c_void_p), ("bg0", C.c_float),
                ("proposal", C.c_int32), ("birth_cdf", C.c_void_p), ("birth_sub", C.c_void_p),
                ("opt_model", C.c_int32), ("sampled_psf", C.c_void_p), ("n_psf", C.c_int32),
                ("psf_slot", C.c_void_p)]


class BatchResults(C.Structure):
    _fields_ = [("map_n", C.c_void_p), ("final_n", C.c_void_p), ("final_state", C.c_void_p),
                ("counters", C.c_void_p), ("n_entries", C.c_void_p), ("status", C.c_void_p),
                ("overflow", C.c_void_p), ("llr_evals", C.c_void_p), ("trace_len", C.c_int32),
                ("n_trace", C.c_void_p), ("x_trace", C.c_void_p), ("pgrid", C.c_void_p), ("pback", C.c_void_p),
                ("grid_stride", C.c_int64), ("grid_ld", C.c_int32), ("grid_slot", C.c_void_p),
                ("pos_trace", C.c_void_p), ("pos_len", C.c_int32), ("pos_thin", C.c_int32),
                ("model_drift", C.c_void_p)]

POS_SLOTS = 32
POS_RECORD = 5 + 3 * POS_SLOTS


# birth proposals of the batched sampler (bamf_roi_batch.proposal)
PROPOSAL = {"reference": 0, "uniform": 1, "learned": 2}


def _check(L, st: int, where: str) -> None:
    if st != abi.BAMF_OK:
        msg = L.bamf_last_error()
        raise abi.BamfError(st, f"{where} ({msg.decode() if msg else ''})")


def crjmcmc_raw(roi: np.ndarray, params: abi.McmcParams, off, sig, back, e0=None,
                rng=(0, 0, 0), scmos=None, arith: str = "exact", record: bool = True,
                grids: bool = True, sampled_psf: np.ndarray | None = None) -> dict:
    """One cRJMCMC call on a (Ysize, Xsize) ROI; raw outputs like oracle.run_chain.
    sampled_psf: a 4-D (P0, P1, P2, P3) array selects OptModel 1 (params.PSFsize
    must hold its shape); None the Gaussian model."""
    L = _declare()
    psf = None
    if sampled_psf is not None:
        psf = np.ascontiguousarray(np.asarray(sampled_psf, np.float32).ravel(order="F"))
        if tuple(params.PSFsize) != tuple(np.shape(sampled_psf)):
            raise ValueError("params.PSFsize must be the sampled PSF's shape")
    ysize, xsize = roi.shape
    data = np.ascontiguousarray(np.asarray(roi, np.float32).ravel(order="F"))
    I, X, Y, BG = e0 if e0 is not None else ([], [], [], 0.0)
    em, keep = abi.make_emitters(len(I), I, X, Y, BG)
    off = np.ascontiguousarray(off, np.float32)
    sig = np.ascontiguousarray(sig, np.float32)
    back = np.ascontiguousarray(back, np.float32)
    sc = None if scmos is None else np.ascontiguousarray(np.asarray(scmos, np.float32).ravel(order="F"))
    r = abi.Rng(*rng)
    steps = int(params.N_Burnin) + int(params.N_Trials)
    chains = None
    if record:
        chains = [abi.alloc_chain(steps, steps * abi.BAMF_NMAX) for _ in range(2)]
    Z = int(params.Grid_Zoom)
    g = xsize * ysize * Z * Z
    pg = np.zeros(g, np.float32) if grids else None
    pb = np.zeros(g, np.float32) if grids else None
    cnt = abi.Counters()
    st = L.bamf_crjmcmc_host_model(
        abi.fptr(data), xsize, ysize, C.byref(em), C.byref(params), abi.fptr(off), off.size,
        abi.fptr(sig), sig.size, abi.fptr(back), back.size, abi.fptr(sc) if sc is not None else None,
        abi.fptr(psf) if psf is not None else None, 1 if psf is not None else 0,
        C.byref(r), ARITH[arith], abi.fptr(pg) if grids else None, abi.fptr(pb) if grids else None,
        C.byref(chains[0][0]) if record else None, C.byref(chains[1][0]) if record else None,
        C.byref(cnt))
    _check(L, st, "bamf_crjmcmc_host_model")
    out = {"counters": cnt.as_dict()}
    if record:
        out["chain"] = abi.chain_to_dict(*chains[0])
        out["chain_test"] = abi.chain_to_dict(*chains[1])
    if grids:
        out["pgrid"] = pg.reshape(xsize * Z, ysize * Z).T.copy()
        out["pback"] = pb.reshape(xsize * Z, ysize * Z).T.copy()
    return out


def crjmcmc_batch_raw(rois: list, params: abi.McmcParams, off, sig, back, e0s=None, seed: int = 0,
                      chain_ids=None, rng_offsets=None, arith: str = "exact", record: bool = True,
                      grids: bool = True, records_per_entry: int = 12) -> list[dict]:
    """Many cRJMCMC calls in one launch (bamf_crjmcmc_batch_host): ROI k is
    rois[k] (Ysize, Xsize), start state e0s[k] = (I, X, Y, BG), stream
    (seed, chain_ids[k], rng_offsets[k]).  Returns one dict per ROI like
    crjmcmc_raw (plus "uniforms_used").  Chains are given
    records_per_entry records per entry of room; a ROI that needs more is
    run again alone with room for BAMF_NMAX (the same stream gives the same
    chain)."""
    L = _declare()
    n = len(rois)
    if n == 0:
        return []
    xs = np.array([r.shape[1] for r in rois], np.int32)
    ys = np.array([r.shape[0] for r in rois], np.int32)
    sizes = xs.astype(np.int64) * ys
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    data = np.ascontiguousarray(np.concatenate([np.asarray(r, np.float32).ravel(order="F") for r in rois]))
    keep = []
    ems = (abi.Emitters * n)()
    for k in range(n):
        I, X, Y, BG = e0s[k] if e0s is not None else ([], [], [], 0.0)
        e, kp = abi.make_emitters(len(I), I, X, Y, BG)
        ems[k] = e
        keep.append(kp)
    pr, arrs = Sampler._priors(off, sig, back)
    cid = None if chain_ids is None else np.ascontiguousarray(chain_ids, np.uint32)
    rof = None if rng_offsets is None else np.ascontiguousarray(rng_offsets, np.uint32)
    steps = int(params.N_Burnin) + int(params.N_Trials)
    chains = None
    if record:
        bufs = [abi.alloc_chain(steps + 1, (steps + 1) * records_per_entry) for _ in range(2 * n)]
        chains = (abi.Chain * (2 * n))(*[b[0] for b in bufs])
    Z = int(params.Grid_Zoom)
    pg = np.zeros(int(sizes.sum()) * Z * Z, np.float32) if grids else None
    pb = np.zeros(int(sizes.sum()) * Z * Z, np.float32) if grids else None
    cnt = (abi.Counters * n)()
    unif = np.zeros(n, np.uint32)
    status = np.zeros(n, np.int32)
    st = L.bamf_crjmcmc_batch_host(
        n, abi.fptr(data), offs.ctypes.data, xs.ctypes.data, ys.ctypes.data, ems, C.byref(params), C.byref(pr),
        None, seed, cid.ctypes.data if cid is not None else None, rof.ctypes.data if rof is not None else None,
        ARITH[arith], abi.fptr(pg) if grids else None, abi.fptr(pb) if grids else None, chains, cnt,
        unif.ctypes.data, status.ctypes.data)
    _check(L, st, "bamf_crjmcmc_batch_host")
    out = []
    for k in range(n):
        if status[k] == abi.BAMF_ERR_CAPACITY and record:
            I, X, Y, BG = e0s[k] if e0s is not None else ([], [], [], 0.0)
            one = crjmcmc_batch_raw([rois[k]], params, off, sig, back, e0s=[(I, X, Y, BG)], seed=seed,
                                    chain_ids=[int(cid[k]) if cid is not None else k],
                                    rng_offsets=[int(rof[k]) if rof is not None else 0], arith=arith,
                                    record=True, grids=grids, records_per_entry=abi.BAMF_NMAX)
            out.append(one[0])
            continue
        if status[k] != abi.BAMF_OK:
            raise abi.BamfError(int(status[k]), f"bamf_crjmcmc_batch_host: ROI {k}")
        d = {"counters": cnt[k].as_dict(), "uniforms_used": int(unif[k])}
        if record:
            d["chain"] = abi.chain_to_dict(chains[2 * k], bufs[2 * k][1])
            d["chain_test"] = abi.chain_to_dict(chains[2 * k + 1], bufs[2 * k + 1][1])
        if grids:
            g0 = int(offs[k]) * Z * Z
            gz = int(sizes[k]) * Z * Z
            d["pgrid"] = pg[g0:g0 + gz].reshape(int(xs[k]) * Z, int(ys[k]) * Z).T.copy()
            d["pback"] = pb[g0:g0 + gz].reshape(int(xs[k]) * Z, int(ys[k]) * Z).T.copy()
        out.append(d)
    return out


def _emitters_of(raw: dict, nn: int):
    """RJMCMCChain::getEmitters (LibRJMCMC.cpp:324-377) on the raw vectors."""
    N = raw["N"]
    n = int(N[nn]) if int(N[nn]) != 0 else 1
    start = int(np.sum(np.maximum(N[:nn], 1)))
    sl = slice(start, start + n)
    return (n, raw["Photons"][sl], raw["X"][sl], raw["Y"][sl], raw["Signal"][sl])


def mex_chain(raw: dict, accepted: dict | None = None) -> list[dict]:
    """Marshal a raw chain into the MEX struct array (cRJMCMC.cpp:159-276):
    one struct per entry except the last; N reported as 0 for the placeholder
    state; the proposed chain takes LLR/PR/JumpType/Accepted from the
    accepted chain (:265-272)."""
    src = accepted if accepted is not None else raw
    out = []
    for nn in range(len(raw["N"]) - 1):
        n, ph, x, y, s = _emitters_of(raw, nn)
        out.append({
            "N": 0.0 if ph[0] == 0 else float(n),
            "X": x.astype(np.float64), "Y": y.astype(np.float64),
            "Photons": ph.astype(np.float64), "Signal": s.astype(np.float64),
            "LLR": float(src["LLR"][nn]), "PR": float(src["PR"][nn]),
            "JumpType": float(src["JumpType"][nn]), "Accepted": float(src["Accepted"][nn]),
            "BG": float(raw["BG"][nn]), "ABG": float(raw["ABG"][nn]), "BBG": float(raw["BBG"][nn]),
        })
    return out


STAT_FIELDS = ["NTrials", "Accept_Jump", "Accept_Split", "Accept_Merge", "Accept_Birth",
               "Accept_Death", "Accept_JumpFg", "Accept_SplitFg", "Accept_MergeFg",
               "Accept_BirthFg", "Accept_DeathFg", "Accept_JumpBg", "Accept_SplitBg",
               "Accept_MergeBg", "Accept_BirthBg", "Accept_DeathBg"]


def mex_stat(counters: dict, params: abi.McmcParams) -> dict:
    """The Stat output (cRJMCMC.cpp:282-305): accept/propose ratios."""
    c = counters
    vals = [float(params.N_Trials) + float(params.N_Burnin)]
    for suf in ("", "Fg", "Bg"):
        for m in ("jump", "split", "merge", "birth", "death"):
            vals.append(c[f"A_{m}{suf}"] / c[f"N_{m}{suf}"])
    return dict(zip(STAT_FIELDS, vals))


def cRJMCMC(Data, E_active: dict, MCMC: abi.McmcParams, Xsize: int, Ysize: int, OffSetPDF,
            SignalPDF, BackPDF, sCMOScorr=None, SampledPSF=None, OptModel: int = 0,
            rng=(0, 0, 0), arith: str = "exact"):
    """The MEX call of rjmcmc.m:102 / mcmc.m:142 with the same five outputs:
    PGrid, PBack, accepted chain, proposed chain, Stat.  OptModel 0 is the
    Gaussian model, 1 the sampled PSF `SampledPSF` (4-D, MATLAB order, its
    shape in MCMC.PSFsize; cRJMCMC.cpp:74); other values are rejected."""
    if OptModel is None:
        OptModel = 0
    if OptModel not in (0, 1):
        raise abi.BamfError(abi.BAMF_ERR_INVALID_ARG, f"cRJMCMC(OptModel={OptModel})")
    psf = None
    if OptModel == 1:
        if SampledPSF is None:
            raise abi.BamfError(abi.BAMF_ERR_INVALID_ARG, "cRJMCMC(OptModel=1) needs SampledPSF")
        psf = np.asarray(SampledPSF, np.float32)
    data = np.asarray(Data, np.float32)[:Ysize, :Xsize]
    e0 = (np.asarray(E_active.get("I", []), np.float32), np.asarray(E_active.get("X", []), np.float32),
          np.asarray(E_active.get("Y", []), np.float32), float(E_active["BG"]))
    raw = crjmcmc_raw(data, MCMC, OffSetPDF, SignalPDF, BackPDF, e0=e0, rng=rng, scmos=sCMOScorr,
                      arith=arith, sampled_psf=psf)
    acc = mex_chain(raw["chain"])
    prop = mex_chain(raw["chain_test"], accepted=raw["chain"])
    return raw["pgrid"], raw["pback"], acc, prop, mex_stat(raw["counters"], MCMC)


def rjmcmc(Data, RJ: RJStruct, Ysize: int, Xsize: int, DriftY: float = 0.0, DriftX: float = 0.0,
           sCMOSVar=None, rng=(0, 0, 0), arith: str = "exact"):
    """@RJ/rjmcmc.m:1-105: empty start, MCMC struct from RJStruct; returns
    (Chain, Stat, PImage, PBackg, ProposedChain)."""
    E = {"N": 0, "I": [], "X": [], "Y": [], "BG": initial_bg(RJ)}
    p = mcmc_params(RJ, DriftX, DriftY)
    pg, pb, acc, prop, stat = cRJMCMC(Data, E, p, Xsize, Ysize, RJ.P_Offset, RJ.P_EmPhotons,
                                      RJ.P_BgEmPhotons, sCMOSVar, rng=rng, arith=arith)
    return acc, stat, pg, pb, prop


def pack_psfs(sampled_psf, params: abi.McmcParams):
    """One sampled PSF (P0, P1, P2, P3) or a stack (n, P0, P1, P2, P3) ->
    (float32 array of the PSFs one after another, each in MATLAB order, n)."""
    a = np.asarray(sampled_psf, np.float32)
    if a.ndim == 4:
        a = a[None]
    if a.ndim != 5 or tuple(a.shape[1:]) != tuple(params.PSFsize):
        raise ValueError("params.PSFsize must be the sampled PSF's shape")
    flat = np.concatenate([np.ravel(x, order="F") for x in a])
    return np.ascontiguousarray(flat), int(a.shape[0])


class BatchGraph:
    """A captured batch (Sampler.capture); keeps its workspace and tensors alive."""

    def __init__(self, sampler, handle, tensors):
        self._s, self._h, self._t = sampler, handle, tensors

    def launch(self, stream=None) -> None:
        L = self._s._L
        _check(L, L.bamf_rjmcmc_batch_graph_launch(self._h, C.c_void_p(stream) if stream else None),
               "bamf_rjmcmc_batch_graph_launch")

    def close(self) -> None:
        if self._h:
            self._s._L.bamf_rjmcmc_batch_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sampler:
    """Batched sampler over device-resident ROIs (torch tensors on cuda)."""

    def __init__(self):
        L = _declare()
        h = C.c_void_p()
        _check(L, L.bamf_workspace_create(C.byref(h)), "bamf_workspace_create")
        self._ws = h
        self._L = L

    def close(self):
        if self._ws:
            self._L.bamf_workspace_destroy(self._ws)
            self._ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _priors(off, sig, back):
        arrs = [np.ascontiguousarray(a, np.float32) for a in (off, sig, back)]
        pr = Priors(abi.fptr(arrs[0]), arrs[0].size, abi.fptr(arrs[1]), arrs[1].size,
                    abi.fptr(arrs[2]), arrs[2].size)
        return pr, arrs

    def run_device(self, dev: dict, params: abi.McmcParams, off, sig, back, seed: int,
                   arith: str = "fast", outs: dict | None = None, stream=None, bg0: float = 0.0,
                   proposal: str = "reference"):
        """dev: dict of torch CUDA tensors data/offsets/xsize/ysize[/psf_sigma,
        scmos, init_n, init_bg, init_ixy, birth_cdf, birth_sub];
        outs: dict of torch CUDA tensors to fill (map_n, final_n, final_state,
        counters, n_entries, status, overflow, llr_evals, and the [n][T]
        traces n_trace (uint8) / x_trace (float32)).  Enqueues on `stream`."""
        pr, keep, b, res = self._structs(dev, params, off, sig, back, outs, bg0, proposal)
        st = self._L.bamf_rjmcmc_batch_device(self._ws, C.byref(b), C.byref(params), C.byref(pr),
                                               int(seed), ARITH[arith], C.byref(res),
                                               C.c_void_p(stream) if stream else None)
        _check(self._L, st, "bamf_rjmcmc_batch_device")

    def capture(self, dev: dict, params: abi.McmcParams, off, sig, back, seed: int, arith: str = "fast",
                outs: dict | None = None, bg0: float = 0.0, proposal: str = "reference") -> "BatchGraph":
        """bamf_rjmcmc_batch_graph_create: the batch of run_device as a CUDA
        graph over the same tensors (one eager run first, then the capture).
        BatchGraph.launch(stream) replays it on whatever the tensors then hold."""
        pr, keep, b, res = self._structs(dev, params, off, sig, back, outs, bg0, proposal)
        h = C.c_void_p()
        _check(self._L, self._L.bamf_rjmcmc_batch_graph_create(self._ws, C.byref(b), C.byref(params), C.byref(pr),
                                                               int(seed), ARITH[arith], C.byref(res), C.byref(h)),
               "bamf_rjmcmc_batch_graph_create")
        return BatchGraph(self, h, (dev, outs))

    def _structs(self, dev, params, off, sig, back, outs, bg0, proposal):
        pr, keep = self._priors(off, sig, back)
        b = RoiBatch()
        b.n_rois = int(dev["xsize"].numel())
        b.side_max = int(dev.get("side_max", 0))
        for k in ("data", "offsets", "xsize", "ysize", "psf_sigma", "scmos", "init_n", "init_bg",
                  "init_ixy", "birth_cdf", "birth_sub", "sampled_psf", "psf_slot"):
            t = dev.get(k)
            setattr(b, k, t.data_ptr() if t is not None else None)
        b.opt_model = 1 if dev.get("sampled_psf") is not None else 0
        b.n_psf = int(dev.get("n_psf", 1))
        b.bg0 = float(bg0)
        b.proposal = PROPOSAL[proposal]
        res = BatchResults()
        outs = outs or {}
        for k in ("map_n", "final_n", "final_state", "counters", "n_entries", "status", "overflow",
                  "llr_evals", "n_trace", "x_trace", "model_drift"):
            t = outs.get(k)
            setattr(res, k, t.data_ptr() if t is not None else None)
        for k in ("pgrid", "pback", "grid_slot", "pos_trace"):
            t = outs.get(k)
            setattr(res, k, t.data_ptr() if t is not None else None)
        res.grid_stride = int(outs.get("grid_stride", 0))
        res.grid_ld = int(outs.get("grid_ld", 0))
        if outs.get("pos_trace") is not None:
            res.pos_len = int(outs["pos_trace"].shape[1])
            res.pos_thin = int(outs.get("pos_thin", 1))
        tr = [outs[k] for k in ("n_trace", "x_trace") if outs.get(k) is not None]
        if tr:
            if any(t.dim() != 2 or t.shape[1] != tr[0].shape[1] for t in tr):
                raise ValueError("n_trace and x_trace must be [n_rois][trace_len] of one length")
            res.trace_len = int(tr[0].shape[1])
        return pr, keep, b, res

    def autotune(self, dev: dict, params: abi.McmcParams, off, sig, back, arith: str = "fast", jumps: int = 200,
                 sample: int = 4864, stream=None, bg0: float = 0.0) -> list:
        """bamf_autotune on a device batch (run_device layout); returns the
        chosen chains per CTA of the 7 size classes (0: class absent)."""
        pr, keep = self._priors(off, sig, back)
        b = RoiBatch()
        b.n_rois = int(dev["xsize"].numel())
        b.side_max = int(dev.get("side_max", 0))
        for k in ("data", "offsets", "xsize", "ysize", "psf_sigma", "scmos", "sampled_psf", "psf_slot"):
            t = dev.get(k)
            setattr(b, k, t.data_ptr() if t is not None else None)
        b.opt_model = 1 if dev.get("sampled_psf") is not None else 0
        b.n_psf = int(dev.get("n_psf", 1))
        b.bg0 = float(bg0)
        L = self._L
        _check(L, L.bamf_autotune(self._ws, C.byref(b), C.byref(params), C.byref(pr), ARITH[arith], int(jumps),
                                  int(sample), C.c_void_p(stream) if stream else None), "bamf_autotune")
        out = (C.c_int32 * 7)()
        _check(L, L.bamf_autotune_result(self._ws, ARITH[arith], out), "bamf_autotune_result")
        return list(out)

    def tuned_shapes(self, arith: str = "fast") -> tuple:
        """(chains per CTA, CTAs per SM of the register budget) per size class."""
        L = self._L
        a, b = (C.c_int32 * 7)(), (C.c_int32 * 7)()
        _check(L, L.bamf_autotune_shapes(self._ws, ARITH[arith], a, b), "bamf_autotune_shapes")
        return list(a), list(b)

    def run_host(self, batch, params: abi.McmcParams, off, sig, back, seed: int,
                 arith: str = "fast", bg0: float = 0.0, init=None, proposal: str = "reference",
                 birth=None, trace_len: int = 0, sampled_psf: np.ndarray | None = None,
                 psf_slot: np.ndarray | None = None, model_drift: bool = False) -> dict:
        """batch: synth.RoiBatch (host numpy); returns numpy results.
        birth: (cdf, sub) host arrays of the LEARNED proposal; trace_len > 0
        adds the n_trace / x_trace outputs; model_drift adds the per-ROI
        largest relative drift of the incremental model (fast arithmetic);
        sampled_psf: a 4-D array of shape
        params.PSFsize, or a stack (n_psf, *PSFsize) with psf_slot[k] naming
        ROI k's, selects the sampled-PSF model (OptModel 1)."""
        pr, keep = self._priors(off, sig, back)
        n = batch.n
        b = RoiBatch()
        b.n_rois = n
        b.side_max = 0
        arrays = {"data": np.ascontiguousarray(batch.data, np.float32),
                  "offsets": np.ascontiguousarray(batch.offsets, np.int64),
                  "xsize": np.ascontiguousarray(batch.xsize, np.int32),
                  "ysize": np.ascontiguousarray(batch.ysize, np.int32),
                  "psf_sigma": np.ascontiguousarray(batch.sigma, np.float32)}
        if init is not None:
            arrays["init_n"] = np.ascontiguousarray(init["n"], np.int32)
            arrays["init_bg"] = np.ascontiguousarray(init["bg"], np.float32)
            arrays["init_ixy"] = np.ascontiguousarray(init["ixy"], np.float32)
        if birth is not None:
            arrays["birth_cdf"] = np.ascontiguousarray(birth[0], np.float32)
            arrays["birth_sub"] = np.ascontiguousarray(birth[1], np.float32)
        if sampled_psf is not None:
            arrays["sampled_psf"], b.n_psf = pack_psfs(sampled_psf, params)
            if psf_slot is not None:
                arrays["psf_slot"] = np.ascontiguousarray(psf_slot, np.int32)
            b.opt_model = 1
        for k, a in arrays.items():
            setattr(b, k, a.ctypes.data)
        b.bg0 = float(bg0)
        b.proposal = PROPOSAL[proposal]
        outs = {"map_n": np.zeros(n, np.int32), "final_n": np.zeros(n, np.int32),
                "final_state": np.zeros((n, FINAL_STRIDE), np.float32),
                "counters": np.zeros((n, 30), np.int32), "n_entries": np.zeros(n, np.int32),
                "status": np.full(n, -1, np.int32), "overflow": np.zeros(n, np.int32),
                "llr_evals": np.zeros(n, np.int32)}
        if trace_len > 0:
            outs["n_trace"] = np.zeros((n, trace_len), np.uint8)
            outs["x_trace"] = np.zeros((n, trace_len), np.float32)
        if model_drift:
            outs["model_drift"] = np.zeros(n, np.float32)
        res = BatchResults()
        for k, a in outs.items():
            setattr(res, k, a.ctypes.data)
        res.trace_len = int(trace_len)
        st = self._L.bamf_rjmcmc_batch_host(self._ws, C.byref(b), C.byref(params), C.byref(pr),
                                             int(seed), ARITH[arith], C.byref(res))
        _check(self._L, st, "bamf_rjmcmc_batch_host")
        return outs
