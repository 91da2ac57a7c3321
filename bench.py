"""Headline benchmark: batched RJMCMC sampler throughput (ROIs/s) on GB300.

Workload (one "step"): the batched uneven-size workload - 100,000 ROIs with
sides uniform over {8,12,16,20,24} px, emitter count ~ Poisson(lambda),
lambda ~ U[0,12], sigma ~ U[1.1,1.5], intensities LogN(ln 1000, 0.4),
background U[5,50], Poisson noise (seeded synthetic data from the
reference forward model) - each ROI run for 3000 burn-in + 3000 trial jumps
with the reference's moves (fast arithmetic), in one persistent launch,
followed by the MAP emitter-count reduction.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value     ROIs/s with inputs resident in HBM (device entry point)
e2e       ROIs/s through bamf_rjmcmc_batch_host with host buffers (H2D/D2H inside)
roofline  the sampler kernel against the measured MUFU log2 rate: one log2 per
          ROI pixel per scored proposal (the likelihood-ratio pass); traffic =
          the DRAM bytes (read + write) of the step's sampler launches measured
          by ncu on this workload (dram__bytes_read.sum + dram__bytes_write.sum),
          given only for that configuration
cpu_baseline  the reference sampler (source/c/LibRJMCMC.cpp compiled unmodified,
          glibc math; the C restatement where that build is absent, and
          beside it where present) on all host cores, on a sample with the
          same number of ROIs of every size class
plain_exact  (rank 0, outside the timed region) the plain-RJMCMC
          configuration (200 ROIs 16x16, 3000+3000 jumps) in exact
          arithmetic, whose chains equal the reference sampler's bit for bit:
          end to end through the host API, throughput at 4,864 ROIs (two
          rounds of the GPU's resident chains), and
          the CPU restatement on the same 200 ROIs with all host threads
frontend  (rank 0, outside the timed region) FindROI + gaussMLE on the
          2000-frame 256x256 front-end workload: frames/s, FindROI against the
          measured HBM bandwidth (one 4-byte read per pixel), fits/s, and an
          end-to-end frames/s with the stack copied from pinned host memory
          and the fits read back (bamf_find_roi_fit_pinned)
dense_e2e (rank 0, outside the timed region) the dense end-to-end frame
          analysis (bamf_gb300.pipeline) on 500 of its frames, 100 per pass:
          frames/s, stage times, localisation RMSE / recall / precision
learned_proposal  (rank 0, outside the timed region) the learned-vs-uniform
          proposal evaluation on 16x16 ROIs (bamf_gb300.learned_eval), 4
          dispersed chains per ROI: network training rate, per-arm chains/s,
          multi-chain bulk ESS/s and R-hat of the emitter count and of the
          mean-X functional, MAP count accuracy, RMSE, and the throughput at
          equal MAP accuracy with RMSE within 5%

Under torchrun (N > 1) every rank runs its own 100,000 ROIs (weak scaling,
no data-path collective); value = all ROIs / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) measured by ncu,
# one pass, on GB300:
#   the five sampler launches of one step of the default workload (100k ROIs,
#   3000+3000 jumps): 159.1 MB read + 294.0 MB written (mostly the per-jump
#   count trace of the MAP summary);
#   the FindROI kernels of one whole-stack call on 600 frames of 256x256
#   (filter, wide maxima, count, scan, emit, crop): 671.2 MB, scaled by frames.
SAMPLER_STEP_DRAM_BYTES = {(100_000, 3000): 453.1e6}
FINDROI_DRAM_BYTES_PER_FRAME = 671.2e6 / 600

METRIC = "RJMCMC ROIs/s (batched sampler, 3000+3000 jumps per ROI)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="bamf", choices=["bamf", "reference"])
    ap.add_argument("--n-rois", type=int, default=100_000)
    ap.add_argument("--jumps", type=int, default=3000)
    ap.add_argument("--cpu-sample", type=int, default=0, help="ROIs per CPU-baseline sample (0: auto)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="launch each size class with the occupancy rule's CTA shape (for profiling)")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-vs-uniform proposal evaluation (16x16 ROIs)")
    ap.add_argument("--learned-train-rois", type=int, default=2_000_000)
    ap.add_argument("--learned-eval-rois", type=int, default=50_000)
    ap.add_argument("--no-frontend", action="store_true", help="skip the FindROI + gaussMLE measurement")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain-RJMCMC exact-arithmetic measurement (200 ROIs 16x16)")
    ap.add_argument("--frontend-frames", type=int, default=2000)
    ap.add_argument("--no-dense", action="store_true", help="skip the dense end-to-end frame analysis")
    ap.add_argument("--dense-frames", type=int, default=500)
    ap.add_argument("--dense-chunk", type=int, default=100, help="frames per pipeline pass of the dense analysis")
    return ap.parse_args()


def dense_bench(n_frames: int, chunk: int = 100) -> dict:
    """The dense end-to-end stress workload on n_frames of its 10,000
    frames (256x256, 100 nm pixels, U[1,10] emitters/um^2, sigma 1.3,
    LogN(ln 800, 0.5), background U[50,200]): priors from the front end,
    16x16 sub-regions (BoxSize 10, Overlap 3), batched sampler with learned
    births (network trained on the generator with this workload's
    statistics), MAP + refinement, stitched posterior image; the stack is
    analysed `chunk` frames per pass (the posterior grids accumulate over
    all passes); frames/s of a warmed run, localisation against the truth."""
    from bamf_gb300 import learned, pipeline, priors, rjstruct, synth
    frames, truth, _ = synth.frames_dense(n_frames, seed=5)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = 3000
    rj.N_BurninMCMC = rj.N_TrialsMCMC = 1000
    rj.SRZoom = 20
    sma = {"MeanPhotons": 800.0, "MinPValue": 0.01, "MinPhotons": 100.0}
    t0 = time.perf_counter()
    priors.findPriors(frames, rj, sma, "No")
    t_priors = time.perf_counter() - t0
    rho = 5.5 * 0.01  # mean emitters per pixel: U[1,10] per um^2, 0.01 um^2 pixels
    rj.Rho = rho
    net = learned.ProposalNet(seed=0)
    t0 = time.perf_counter()
    net.train(1000, batch=1024, lr=2e-3, data_seed=9, mean_n=rho * 256, i_median=800.0, i_logsd=0.5,
              bg=50.0, bg_max=200.0)
    t_train = time.perf_counter() - t0
    pipeline.analyze_frames(frames[:, :, :2], rj, proposal="learned", net=net, seed=2)  # warm-up
    out = pipeline.analyze_frames(frames, rj, proposal="learned", net=net, seed=2, chunk_frames=chunk)
    st = pipeline.localisation_stats(out["ClustInfo"], truth)
    t = out["timing"]
    return {"workload": f"dense end to end: {n_frames} frames 256x256, U[1,10] emitters/um^2, 16x16 sub-regions "
                        f"(BoxSize 10, Overlap 3), learned births, 3000+3000 jumps + 1000+1000 refinement, "
                        f"{chunk} frames per pass",
            "frames_per_s": n_frames / t["total"], "subregions": out["n_subregions"],
            "subregions_per_s": out["n_subregions"] / t["total"],
            "stage_seconds": {k: round(v, 4) for k, v in t.items()},
            "priors_seconds": t_priors, "network_train_seconds": t_train, **st}


def measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s (of fallback)"


def plain_exact_bench(n_large: int = 4864) -> dict:
    """The plain-RJMCMC configuration (200 ROIs of 16x16, 3000+3000 jumps,
    the reference proposal) in exact arithmetic, the path whose chains equal
    the reference sampler's bit for bit: the 200-ROI batch end to end through
    the host API, the same generator at n_large ROIs for throughput (device
    inputs), and the CPU restatement (bit-identical to the reference build)
    on all host threads over the 200 ROIs."""
    import torch

    from bamf_gb300 import rjstruct, sampler, synth
    rj = rjstruct.c0_rjstruct()
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    s = sampler.Sampler()
    out = {"workload": "plain RJMCMC, exact arithmetic: 200 ROIs 16x16, 3000+3000 jumps (and the same "
                       f"generator at {n_large} ROIs)"}
    b = synth.roi_batch_c0(200, seed=0)
    s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=7, arith="exact", bg0=bg0)
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=7, arith="exact", bg0=bg0)
    out["seconds_200"] = time.perf_counter() - t
    out["rois_per_s_200_e2e"] = 200 / out["seconds_200"]
    assert (r["status"] == 0).all()
    bl = synth.roi_batch_c0(n_large, seed=1)
    dev = {"data": torch.from_numpy(bl.data).cuda(), "offsets": torch.from_numpy(bl.offsets).cuda(),
           "xsize": torch.from_numpy(bl.xsize).cuda(), "ysize": torch.from_numpy(bl.ysize).cuda(),
           "psf_sigma": torch.from_numpy(bl.sigma).cuda(), "side_max": 16}
    outs = {k: torch.zeros(n_large, dtype=torch.int32, device="cuda") for k in ("map_n", "status")}
    s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=7, arith="exact", outs=outs, bg0=bg0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=7, arith="exact", outs=outs, bg0=bg0)
    e1.record()
    torch.cuda.synchronize()
    out["rois_per_s_large"] = n_large / (e0.elapsed_time(e1) * 1e-3)
    threads = os.cpu_count() or 1
    kind = cpu_kind()
    rate, secs, _ = cpu_sample_rate(b, rj, p, bg0, 200, threads, kind)
    out["cpu_rois_per_s_200"] = rate
    out["cpu_kind"] = CPU_DESC[kind][0]
    out["cpu_cores"] = threads
    out["cpu_seconds_200"] = secs
    return out


def gaussmle_flops_per_fit(sz: int, iterations: int) -> int:
    """Algorithmic FP32 operations of one 'Basic' fit (an FMA counted as 2,
    a transcendental or a reciprocal as 1): the start-up filter (sz^2
    positions x sz^2 weighted pixels, 3 each, plus the division), every
    Newton iteration (per pixel 25: model 3, derivatives 5, the Poisson
    factors 5, the four num/den sums 12; per axis value 2 erf + 2 exp + 16)
    and the Fisher information (per pixel 30) plus the 4 x 4 inversion."""
    px = sz * sz
    return px * px * 3 + px + iterations * (px * 25 + 2 * sz * 20) + px * 30 + 100


def frontend_bench(n_frames: int, steps: int = 5, warmup: int = 3, fp32_peak: float | None = None) -> dict:
    """FindROI + gaussMLE on n_frames 256x256 frames (Poisson(50) emitters
    per frame, sigma 1.3, I ~ LogN(ln 1500, 0.3), bg 20; Boxsize 7, Minval
    from findROI.m:74, 10 Newton iterations).  The stack (524 MB at 2000
    frames) is larger than L2, so no flush between calls."""
    import torch

    from bamf_gb300 import frontend, synth
    stack, _ = synth.frames(n_frames, seed=3)
    host = torch.from_numpy(np.asfortranarray(stack).ravel(order="F")).pin_memory()
    dev = host.cuda()
    n = dev.numel()
    mv = frontend.default_minval()
    fr = frontend.FindRoiDevice()
    ev = lambda: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))  # noqa: E731
    for _ in range(warmup):
        out = fr.run(dev, 256, 256, n_frames, boxsize=7, minval=mv)
    torch.cuda.synchronize()
    t_find = []
    for _ in range(steps):
        e0, e1 = ev()
        e0.record()
        out = fr.run(dev, 256, 256, n_frames, boxsize=7, minval=mv)
        e1.record()
        torch.cuda.synchronize()
        t_find.append(e0.elapsed_time(e1) * 1e-3)
    count = int(out["count"].item())
    rois = out["stack"][:count].contiguous()
    for _ in range(warmup):
        frontend.gauss_mle_device(rois, 7, count, 1.3, 10)
    torch.cuda.synchronize()
    t_mle = []
    for _ in range(steps):
        e0, e1 = ev()
        e0.record()
        frontend.gauss_mle_device(rois, 7, count, 1.3, 10)
        e1.record()
        torch.cuda.synchronize()
        t_mle.append(e0.elapsed_time(e1) * 1e-3)
    # end to end through the API for host frames: pinned frames in (copied
    # in chunks; each chunk's filters start as it lands, and its maxima are
    # compacted, cropped and fitted while later chunks are copied), fits out
    e2e = []
    dframes = torch.empty_like(dev)
    for _ in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        o = fr.run_fit_pinned(host, 256, 256, n_frames, boxsize=7, minval=mv, psf_sigma=1.3, iterations=10,
                              capacity=max(1024, n // 256), dev_frames=dframes)
        c = int(o["count"].item())
        res = (o["coords"][:c].cpu(), o["P"][:, :c].cpu(), o["CR"][:, :c].cpu(), o["LL"][:c].cpu())
        e2e.append(time.perf_counter() - t0)
    d2h = sum(r.numel() * r.element_size() for r in res)
    tf, tm = statistics.median(t_find), statistics.median(t_mle)
    peak, src = measured_hbm_gbs()
    alg = 4.0 * n + count * (3 + 2 + 49) * 4.0
    return {
        "workload": f"FindROI + gaussMLE: {n_frames} frames 256x256, Boxsize 7, 10 iterations",
        "findroi_ms": tf * 1e3, "findroi_frames_per_s": n_frames / tf,
        "findroi_roofline": {"bound": "hbm", "achieved": alg / tf / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": alg / tf / 1e9 / peak, "traffic": FINDROI_DRAM_BYTES_PER_FRAME * n_frames,
                             "traffic_note": "DRAM bytes of a 600-frame call measured by ncu, scaled by frames",
                             "peak_source": src,
                             "algorithmic_bytes": alg},
        "maxima": count, "gaussmle_ms": tm * 1e3, "gaussmle_fits_per_s": count / tm,
        "gaussmle_achieved_gbs": count * (49 + 9) * 4.0 / tm / 1e9,
        "gaussmle_roofline": None if not fp32_peak else {
            "bound": "fp32 issue", "achieved": count * gaussmle_flops_per_fit(7, 10) / tm / 1e12,
            "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
            "frac": count * gaussmle_flops_per_fit(7, 10) / tm / fp32_peak,
            "flops_per_fit": gaussmle_flops_per_fit(7, 10),
            "peak_source": "FP32 FMA rate measured in-process by bamf_probe_peaks"},
        "e2e": {"value": n_frames / statistics.median(e2e[1:]), "unit": "frames/s",
                "h2d_bytes_per_step": int(host.numel() * 4), "d2h_bytes_per_step": int(d2h),
                "calls": len(e2e) - 1,
                "seconds_per_call": {"median": statistics.median(e2e[1:]), "min": min(e2e[1:]),
                                     "max": max(e2e[1:])}},
    }


def noalloc_bench(s, dev, outs, p, rj, bg0, n, stream) -> dict:
    """One call each of the workspace entry point and the allocation-free
    one on the bench batch, without MAP counts (the MAP trace of this batch
    is beyond the allocation-free scratch), timed with CUDA events; the
    per-ROI outputs must agree."""
    import ctypes as C

    import torch

    from bamf_gb300 import abi, sampler
    L = sampler._declare()
    L.bamf_rjmcmc_batch_device_noalloc.restype = C.c_int
    L.bamf_rjmcmc_batch_device_noalloc.argtypes = [
        C.POINTER(sampler.RoiBatch), C.POINTER(abi.McmcParams), C.POINTER(sampler.Priors),
        C.c_uint32, C.c_int, C.POINTER(sampler.BatchResults), C.c_void_p]
    o1 = {k: torch.zeros(n, dtype=torch.int32, device="cuda") for k in ("final_n", "status")}
    o2 = {k: torch.zeros(n, dtype=torch.int32, device="cuda") for k in ("final_n", "status")}
    ev = lambda: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))  # noqa: E731
    a0, a1 = ev()
    a0.record(stream)
    s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=77, arith="fast", outs=o1,
                 stream=stream.cuda_stream, bg0=bg0)
    a1.record(stream)
    pr, keep, bs, rs = s._structs(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, o2, bg0, "reference")
    b0, b1 = ev()
    b0.record(stream)
    st = L.bamf_rjmcmc_batch_device_noalloc(C.byref(bs), C.byref(p), C.byref(pr), 77, abi.BAMF_ARITH_FAST,
                                            C.byref(rs), C.c_void_p(stream.cuda_stream))
    b1.record(stream)
    torch.cuda.synchronize()
    abi.check(st, "bamf_rjmcmc_batch_device_noalloc")
    same = bool(torch.equal(o1["final_n"], o2["final_n"]) and torch.equal(o1["status"], o2["status"]))
    tw, tn = a0.elapsed_time(a1) * 1e-3, b0.elapsed_time(b1) * 1e-3
    return {"workspace_rois_per_s": n / tw, "noalloc_rois_per_s": n / tn, "same_results": same,
            "note": "no MAP counts in either; size classes serial on one stream in the allocation-free call"}


def workload_label(n_rois: int, jumps: int) -> str:
    return (f"batched uneven RJMCMC: {n_rois // 1000}k ROIs, sides {{8,12,16,20,24}} px, "
            f"{jumps}+{jumps} jumps")


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(n_rois: int, seed: int, jumps: int):
    from bamf_gb300 import rjstruct, synth
    b = synth.roi_batch_uneven(n_rois, seed=seed)
    rj = rjstruct.uneven_rjstruct()
    rj.N_Burnin = rj.N_Trials = jumps
    return b, rj, rjstruct.mcmc_params(rj), rjstruct.initial_bg(rj)


def cpu_kind() -> str:
    """The reference sampler itself (source/c/LibRJMCMC.cpp compiled
    unmodified, glibc math) when its build is available, else the C
    restatement (glibc math, bit-identical outputs)."""
    import oracle
    oracle.build()
    return "ref_native" if oracle.available("ref_native") else "port_native"


def stratified(b, per_class: int, start: int = 0):
    """The ROIs [start, start + per_class) of every size class of batch b,
    interleaved class by class (the CPU sample covers all sides equally)."""
    from bamf_gb300 import synth
    sides = np.maximum(b.xsize, b.ysize)
    cols = [np.flatnonzero(sides == sd)[start:start + per_class] for sd in np.unique(sides)]
    idx = np.stack([c[:min(len(x) for x in cols)] for c in cols], 1).ravel()
    return synth.RoiBatch(data=b.data, offsets=b.offsets[idx], xsize=b.xsize[idx], ysize=b.ysize[idx],
                          sigma=b.sigma[idx], bg=b.bg[idx], true_n=b.true_n[idx], true_x=[], true_y=[],
                          true_i=[])


def cpu_sample_rate(b, rj, p, bg0, n_sample: int, threads: int, kind: str = "port_native", per_class=None):
    """A CPU sampler (`kind`: the reference build "ref_native" or the C
    restatement "port_native") on a sample of batch b, all `threads` host
    threads: the first n_sample ROIs, or per_class ROIs of every size class;
    returns (ROIs/s, seconds, ROIs)."""
    import oracle
    from bamf_gb300 import synth
    if per_class:
        sub = stratified(b, per_class)
    else:
        sub = synth.RoiBatch(
            data=b.data, offsets=b.offsets[:n_sample], xsize=b.xsize[:n_sample],
            ysize=b.ysize[:n_sample], sigma=b.sigma[:n_sample], bg=b.bg[:n_sample],
            true_n=b.true_n[:n_sample], true_x=[], true_y=[], true_i=[])
    t = time.perf_counter()
    oracle.run_batch(sub, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, bg0, seed=1,
                     threads=threads, kind=kind)
    dt = time.perf_counter() - t
    return sub.n / dt, dt, sub.n


CPU_DESC = {"ref_native": ("reference", "the reference sampler source/c/LibRJMCMC.cpp compiled unmodified "
                                        "(glibc math) behind the project's cRJMCMC driver"),
            "port_native": ("port", "glibc-math C restatement, bit-identical to the reference sampler build")}


def run_reference(a, rank, world):
    if rank != 0:
        return
    b, rj, p, bg0 = workload(a.n_rois, 2, a.jumps)
    threads = os.cpu_count() or 1
    kind = cpu_kind()
    per_class = a.cpu_sample or max(2 * threads, 8)  # 5 classes x 2 per thread: ~2 s per step on 16 cores
    for _ in range(a.warmup):
        cpu_sample_rate(b, rj, p, bg0, 0, threads, kind, per_class=max(per_class // 8, 1))
    rates, secs = [], []
    n = 0
    for _ in range(a.steps):
        r, s, n = cpu_sample_rate(b, rj, p, bg0, 0, threads, kind, per_class=per_class)
        rates.append(r)
        secs.append(s)
    v = len(rates) * n / sum(secs)
    ck, desc = CPU_DESC[kind]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "ROIs/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, reference forward model + Poisson noise)",
        "config": {"workload": workload_label(a.n_rois, a.jumps), "n_rois": a.n_rois,
                   "jumps": [a.jumps, a.jumps], "parallelism": "host threads", "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "ROIs/s", "cores": threads, "kind": ck,
                         "sample": f"{n} ROIs per step: the first {per_class} of each size class of the "
                                   f"workload (same seeds); {desc}"},
        "e2e": {"value": v, "unit": "ROIs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        return run_reference(a, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from bamf_gb300 import abi, build, sampler
    build.build()
    import ctypes as C
    L = abi.lib()
    L.bamf_probe_peaks.restype = C.c_int
    L.bamf_probe_peaks.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]

    from bamf_gb300 import replicas
    b, rj, p, bg0 = workload(a.n_rois, replicas.rank_seed(2, rank), a.jumps)
    dev = {
        "data": torch.from_numpy(b.data).cuda(), "offsets": torch.from_numpy(b.offsets).cuda(),
        "xsize": torch.from_numpy(b.xsize).cuda(), "ysize": torch.from_numpy(b.ysize).cuda(),
        "psf_sigma": torch.from_numpy(b.sigma).cuda(), "side_max": int(max(b.xsize.max(), b.ysize.max())),
    }
    n = b.n
    outs = {"map_n": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "final_n": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "status": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "llr_evals": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "overflow": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "n_entries": torch.zeros(n, dtype=torch.int32, device="cuda")}
    s = sampler.Sampler()
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1234, arith="fast",
                     outs=outs, stream=stream.cuda_stream, bg0=bg0)

    # CTA shape per size class by the project's autotuner (short chains on a sample of each class)
    if a.no_autotune:
        tuned = budget = "occupancy rule"
    else:
        tuned = s.autotune(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, arith="fast", jumps=400,
                           sample=4864, stream=stream.cuda_stream, bg0=bg0)
        budget = s.tuned_shapes("fast")[1]
    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    assert int((outs["status"] != 0).sum()) == 0, "sampler reported ROI errors"

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with Clocks(local) as clk:
        for _ in range(a.steps):
            flush.fill_(1.0)  # L2 flush between timed steps (outside the events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    total = replicas.max_over_ranks(sum(times), dist, "cuda")
    value = replicas.whole_job_rate(a.steps * n, world, total)
    step_s = total / a.steps

    # roofline: one MUFU log2 per ROI pixel per scored proposal
    llr = outs["llr_evals"].to(torch.int64).cpu().numpy()
    npix = (b.xsize.astype(np.int64) * b.ysize.astype(np.int64))
    lg2_per_step = float((llr * npix).sum())
    achieved = lg2_per_step / step_s
    fp32 = C.c_double()
    mufu = C.c_double()
    abi.check(L.bamf_probe_peaks(C.byref(fp32), C.byref(mufu)), "bamf_probe_peaks")

    e2e = None
    if not a.no_e2e:
        host_out = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1234,
                              arith="fast", bg0=bg0)  # warm
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        calls = []
        for _ in range(5):
            t0 = time.perf_counter()
            host_out = s.run_host(b, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=1234,
                                  arith="fast", bg0=bg0)
            calls.append(replicas.max_over_ranks(time.perf_counter() - t0, dist, "cuda"))
        dt = statistics.median(calls)
        h2d = b.data.nbytes + b.offsets.nbytes + b.xsize.nbytes + b.ysize.nbytes + b.sigma.nbytes
        d2h = sum(v.nbytes for v in host_out.values())
        e2e = {"value": replicas.whole_job_rate(n, world, dt), "unit": "ROIs/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "calls": len(calls),
               "seconds_per_call": {"median": dt, "min": min(calls), "max": max(calls)}}

    # the allocation-free entry point against the workspace one, both
    # without MAP counts (the MAP trace of 100k ROIs is beyond the fixed scratch)
    noalloc_block = None
    if rank == 0:
        noalloc_block = noalloc_bench(s, dev, outs, p, rj, bg0, n, stream)

    # per step: photon_bucket_kernel and order_kernel (the batch order), one sampler launch per
    # non-empty size class, map_n_kernel
    sides = np.maximum(b.xsize, b.ysize)
    bounds = [8, 12, 16, 20, 24, 28, 32]
    classes = {next(i for i, hi in enumerate(bounds) if sd <= hi) for sd in np.unique(sides)}
    launches_per_step = 3 + len(classes)

    learned_block = None
    if rank == 0 and not a.no_learned:
        from bamf_gb300 import learned_eval
        r = learned_eval.evaluate(train_rois=a.learned_train_rois, n_eval=a.learned_eval_rois)
        arms = r["arms"]
        learned_block = {
            "workload": r["workload"],
            "train_rois_per_s": r["train_rois_per_s"], "infer_seconds": r["infer_seconds"],
            **{f"{k}_{f}": arms[k][f] for k in arms for f in
               ("chains_per_s", "ess_n_per_chain", "ess_x_per_chain", "ess_n_per_s", "ess_x_per_s",
                "rhat_n_median", "rhat_x_median", "rhat_n_above_1_05", "rhat_x_above_1_05",
                "map_count_accuracy", "rmse_px")},
            "ess_n_per_s_ratio": r["ess_n_per_s_ratio"], "ess_x_per_s_ratio": r["ess_x_per_s_ratio"],
            "ess_n_per_s_ratio_init": r["ess_n_per_s_ratio_init"],
            "ess_x_per_s_ratio_init": r["ess_x_per_s_ratio_init"],
            "equal_accuracy": r["equal_accuracy_vs_uniform_at_full_length"],
            "accuracy_vs_jumps": r["accuracy_vs_jumps"],
        }

    plain_block = None
    if rank == 0 and not a.no_plain:
        plain_block = plain_exact_bench()

    frontend_block = None
    if rank == 0 and not a.no_frontend:
        frontend_block = frontend_bench(a.frontend_frames, fp32_peak=fp32.value)
    dense_block = None
    if rank == 0 and not a.no_dense:
        dense_block = dense_bench(a.dense_frames, a.dense_chunk)

    cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        per_class = a.cpu_sample or max(2 * threads, 8)  # ~30 thread-seconds of CPU work
        kind = cpu_kind()
        rate, secs, ns = cpu_sample_rate(b, rj, p, bg0, 0, threads, kind, per_class=per_class)
        ck, desc = CPU_DESC[kind]
        cpu = {"value": rate, "unit": "ROIs/s", "cores": threads, "kind": ck,
               "sample": f"{ns} ROIs: the first {per_class} of each size class of the workload, {secs:.1f} s "
                         f"on {threads} host threads; {desc}"}
        if kind != "port_native":
            prate, psecs, _ = cpu_sample_rate(b, rj, p, bg0, 0, threads, "port_native", per_class=per_class)
            cpu["port_value"] = prate
            cpu["port"] = CPU_DESC["port_native"][1]

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "ROIs/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, reference forward model + Poisson noise)",
            "config": {"workload": workload_label(n, a.jumps), "n_rois": n, "jumps": [a.jumps, a.jumps],
                       "arith": "fast", "parallelism": f"replicas x{world}",
                       "l2": "flushed between timed steps (512 MB write)",
                       "chains_per_cta_by_size_class": tuned,
                       "ctas_per_sm_register_budget_by_size_class": budget},
            "roofline": {"bound": "sfu", "achieved": achieved / 1e9, "peak": mufu.value / 1e9,
                         "unit": "Gop/s (MUFU log2)", "frac": achieved / mufu.value,
                         "traffic": SAMPLER_STEP_DRAM_BYTES.get((a.n_rois, a.jumps)),
                         "traffic_unit": "bytes per step (all sampler launches)",
                         "peak_source": "measured in-process by bamf_probe_peaks (MUFU lg2 probe)",
                         "fp32_peak_tflops_measured": fp32.value / 1e12},
            "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches_per_step * a.steps,
            "clocks": clk.summary(),
            "learned_proposal": learned_block,
            "plain_exact": plain_block,
            "frontend": frontend_block,
            "dense_e2e": dense_block,
            "noalloc": noalloc_block,
            "overflow_rois_frac": float((outs["overflow"] > 0).float().mean().item()),
            "map_n_mean": float(outs["map_n"].float().mean().item()),
            "true_n_mean": float(b.true_n.mean()),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
