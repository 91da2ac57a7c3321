"""The reference's frame analysis (@RJ/RJ.m:185-256 with analyzeROIs.m,
findMap.m, mcmc.m, removeOverlapping.m, stitchROIs.m) as one GPU pipeline:

  frames -> sub-regions (makeSubRegions, packed for the sampler)
         -> [learned birth tables: network inference on the 16x16 tiles,
             uniform tables for the smaller edge tiles]
         -> batched sampler, posterior grids accumulated per sub-region
            position over frames (analyzeROIs.m:153), thinned state trace
         -> MAP count + k-means (findMap), fixed-count refinement (mcmc)
         -> emitters in frame coordinates, those in another sub-region's
            interior dropped (mcmc.m:43-71, 175-199)
         -> overlap removal and stitching of the posterior grids

Frames are (Y, X, Z) in MATLAB orientation.  `analyze_frames` returns the
ClustInfo-like localisations, the stitched posterior image and a timing
breakdown (CUDA-synchronised wall time per stage).
"""
from __future__ import annotations

import time

import numpy as np

from . import learned, mapfit, rjstruct, sampler, tiles


def _sync():
    import torch
    torch.cuda.synchronize()


def uniform_fill(cdf, sub, xsize, ysize, tile: int):
    """Uniform birth tables for the ROIs that are not tile x tile (the
    network sees only full tiles)."""
    import torch
    n = int(xsize.numel())
    npix = (xsize * ysize).to(torch.int64)
    edge = torch.nonzero(npix != tile * tile).flatten()
    if edge.numel() == 0:
        return
    c = cdf.view(n, tile * tile)
    p = torch.arange(tile * tile, device=cdf.device, dtype=torch.float32)
    ne = npix.index_select(0, edge).to(torch.float32)
    vals = torch.clamp((p[None, :] + 1.0) / ne[:, None], max=1.0)
    c.index_copy_(0, edge, vals)
    sub.view(n, tile * tile, 16).index_fill_(0, edge, 1.0 / 16.0)


def global_emitters(rec: dict, roi_ind, xsize, ysize, frame_num, xsub: int, ysub: int, box: int, overlap: int):
    """mcmc.m:43-71, 175-199: emitters of every ROI in frame coordinates,
    dropping those at or before the interior's start or past its end."""
    X, Y, I = rec["X"], rec["Y"], rec["I"]
    K = rec["N"]
    n = len(K)
    ind = np.asarray(roi_ind)
    ix = (ind - 1) // xsub + 1          # mcmc.m uses Xsub for both (square frames)
    iy = ind - (ix - 1) * xsub
    xs, ys = np.asarray(xsize), np.asarray(ysize)
    bx = np.where(ix != 1, overlap, 0)
    by = np.where(iy != 1, overlap, 0)
    ex = np.where(ix != xsub, xs - overlap, xs)
    ey = np.where(iy != ysub, ys - overlap, ys)
    slot = np.arange(X.shape[1])[None, :]
    valid = slot < K[:, None]
    keep = valid & (X > bx[:, None]) & (X <= ex[:, None]) & (Y > by[:, None]) & (Y <= ey[:, None])
    gx = X + ((ix - 1) * box - bx)[:, None]
    gy = Y + ((iy - 1) * box - by)[:, None]
    fr = np.broadcast_to(np.asarray(frame_num)[:, None], X.shape)
    out = {"X": gx[keep], "Y": gy[keep], "I": I[keep], "X_SE": rec["X_SE"][keep], "Y_SE": rec["Y_SE"][keep],
           "I_SE": rec["I_SE"][keep], "FrameNum": fr[keep], "ROInum": np.broadcast_to(np.arange(n)[:, None],
                                                                                         X.shape)[keep]}
    return out


def match(found_x, found_y, true_x, true_y, radius: float = 1.0):
    """Greedy one-to-one matching of found to true positions within
    `radius` (closest pairs first); returns [pairs][3]: squared distance,
    dx, dy (found - true)."""
    from scipy.spatial import cKDTree
    if len(found_x) == 0 or len(true_x) == 0:
        return np.zeros((0, 3))
    t = cKDTree(np.c_[true_x, true_y])
    pairs = t.query_ball_point(np.c_[found_x, found_y], r=radius)
    cand = [((found_x[i] - true_x[j]) ** 2 + (found_y[i] - true_y[j]) ** 2, i, j)
            for i, js in enumerate(pairs) for j in js]
    cand.sort()
    uf, ut, d2 = set(), set(), []
    for d, i, j in cand:
        if i in uf or j in ut:
            continue
        uf.add(i)
        ut.add(j)
        d2.append((d, found_x[i] - true_x[j], found_y[i] - true_y[j]))
    return np.array(d2).reshape(-1, 3)


def analyze_frames(frames: np.ndarray, rj, box: int = 10, overlap: int = 3, proposal: str = "learned",
                   net=None, seed: int = 1, pos_len: int = 200, grids: bool = True, sampled_psf=None,
                   chunk_frames: int | None = None) -> dict:
    """Frames (Y, X, Z) -> sub-regions -> sampler + MAP + refinement ->
    stitched posterior image and global emitter list.  sampled_psf: None
    (Gaussian PSF), one 4-D sampled PSF, or one per sub-region position
    (psf.find_psf_sma's list), selects OptModel 1 (analyzeROIs.m:142-146).
    chunk_frames: analyse the stack chunk_frames frames at a time (device
    memory for the chain traces stays bounded; the posterior grids of each
    sub-region position accumulate over all chunks, as over all frames in
    analyzeROIs.m:153), then stitch once.  Every chunk's sampler streams
    are keyed by its first frame, so chunking changes which uniforms a
    sub-region's chain draws but not its law."""
    import torch
    Y, X, Z = frames.shape
    T = box + 2 * overlap
    Zm = int(rj.SRZoom)
    Tz = Zm * T
    chunk = Z if not chunk_frames else max(1, min(int(chunk_frames), Z))
    timing = {"h2d": 0.0, "subregions": 0.0, "network": 0.0, "sampler_map_refine": 0.0}
    extra = None
    cis, map_ns, n_total, geom = [], [], 0, None
    for f0 in range(0, Z, chunk):
        part = frames[:, :, f0:f0 + chunk]
        zc = part.shape[2]
        _sync()
        t0 = time.perf_counter()
        dev_frames = torch.from_numpy(np.asfortranarray(part, np.float32).ravel(order="F")).cuda()
        _sync()
        timing["h2d"] += time.perf_counter() - t0
        t = time.perf_counter()
        sr = tiles.make_subregions_device(dev_frames, Y, X, zc, box, overlap, packed=True)
        dev = {"data": sr["data"], "offsets": sr["offsets"], "xsize": sr["xsize"], "ysize": sr["ysize"],
               "side_max": T}
        _sync()
        timing["subregions"] += time.perf_counter() - t
        n = sr["n"]
        n_total += n
        if proposal == "learned":
            if T != learned.SIDE:
                raise ValueError("the learned proposal needs 16x16 sub-regions (box + 2 overlap = 16)")
            t = time.perf_counter()
            tab = net.infer(sr["data"].view(n, T * T))
            uniform_fill(tab["cdf"], tab["sub"], sr["xsize"], sr["ysize"], T)
            dev["birth_cdf"], dev["birth_sub"] = tab["cdf"], tab["sub"]
            _sync()
            timing["network"] += time.perf_counter() - t
        per = sr["Xsub"] * sr["Ysub"]
        if geom is None:
            geom = {k: sr[k][:per].contiguous() for k in ("xsize", "ysize", "roi_ind", "frame_num")}
            geom.update(Xsub=sr["Xsub"], Ysub=sr["Ysub"], per=per)
            if grids:
                extra = {"pgrid": torch.zeros(per * Tz * Tz, dtype=torch.float32, device="cuda"),
                         "pback": torch.zeros(per * Tz * Tz, dtype=torch.float32, device="cuda"),
                         "grid_stride": Tz * Tz, "grid_ld": Tz}
        if extra is not None:
            extra["grid_slot"] = (sr["roi_ind"] - 1).contiguous()
        t = time.perf_counter()
        psf_kw = {}
        if sampled_psf is not None:
            stack = np.asarray(sampled_psf, np.float32)
            psf_kw["sampled_psf"] = stack
            if stack.ndim == 5:
                if stack.shape[0] != per:
                    raise ValueError("one sampled PSF per sub-region position is needed")
                psf_kw["psf_slot"] = (sr["roi_ind"] - 1).to(torch.int32).contiguous()
        res = mapfit.analyze(dev, rj, seed=seed + f0, proposal=proposal, pos_len=pos_len, grids=extra, **psf_kw)
        _sync()
        timing["sampler_map_refine"] += time.perf_counter() - t
        rec = res["refined"]
        ci = global_emitters(rec, sr["roi_ind"].cpu().numpy(), sr["xsize"].cpu().numpy(),
                             sr["ysize"].cpu().numpy(), sr["frame_num"].cpu().numpy() + f0, sr["Xsub"], sr["Ysub"],
                             box, overlap)
        ci["ROInum"] = ci["ROInum"] + (n_total - n)
        cis.append(ci)
        map_ns.append(res["map_n"])
        del dev_frames, sr, dev, res
    out = {"n_subregions": n_total, "timing": timing}
    t = time.perf_counter()
    if grids:
        # one grid per sub-region position, summed over frames; frame 1's ROI_Struct rows describe them
        per = geom["per"]
        for key, name in (("pgrid", "PImage"), ("pback", "PBg")):
            g = extra[key]
            tiles.remove_overlapping_device(g, per, Tz, geom["xsize"], geom["ysize"], geom["roi_ind"],
                                            geom["Xsub"], geom["Ysub"], overlap, Zm)
            img, bad = tiles.stitch_rois_device(g, per, Tz, geom["xsize"], geom["ysize"], geom["frame_num"],
                                                geom["roi_ind"], (Y, X, 1), box, overlap, Zm)
            out[name] = img.view(Zm * X, Zm * Y).t()
    _sync()
    timing["stitch"] = time.perf_counter() - t
    out["ClustInfo"] = {k: np.concatenate([c[k] for c in cis]) for k in cis[0]}
    out["map_n"] = map_ns[0] if len(map_ns) == 1 else _cat(map_ns)
    timing["total"] = sum(timing.values())
    return out


def _cat(parts):
    import torch
    if isinstance(parts[0], torch.Tensor):
        return torch.cat(parts)
    return np.concatenate(parts)


def localisation_stats(ci: dict, truth, radius: float = 1.0) -> dict:
    """RMSE of matched pairs, recall and precision against per-frame truth
    [(X, Y, I), ...] (0-based frame k = FrameNum - 1)."""
    pairs, nt, nf = [], 0, 0
    fn = np.asarray(ci["FrameNum"])
    for k, (tx, ty, _) in enumerate(truth):
        sel = fn == k + 1
        pairs.append(match(ci["X"][sel], ci["Y"][sel], tx, ty, radius))
        nt += len(tx)
        nf += int(sel.sum())
    P = np.concatenate(pairs) if pairs else np.zeros((0, 3))
    m = len(P)
    return {"rmse_px": float(np.sqrt(P[:, 0].mean())) if m else float("nan"), "recall": m / max(nt, 1),
            "precision": m / max(nf, 1), "matched": m, "true": nt, "found": nf,
            "bias_x": float(P[:, 1].mean()) if m else float("nan"),
            "bias_y": float(P[:, 2].mean()) if m else float("nan")}
