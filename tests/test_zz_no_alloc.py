"""The allocation-free sampler entry point (bamf_rjmcmc_batch_device_noalloc)
against the workspace entry point (bamf_rjmcmc_batch_device).

Callers that cannot allocate device memory - hosts whose own pool owns the
GPU memory (MATLAB's gpuArray allocator, a framework's caching allocator),
latency-bound loops that cannot take cudaMalloc's synchronisation - use the
variant whose scratch is a fixed array inside the library.  Both entry points run the same kernels on
the same uniform streams, so every per-ROI result must be identical; the
variant is called twice in a row to show that the shared scratch carries
nothing from one call into the next.  This file is collected last so that a
run stopping at its first failure has run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OUT_FIELDS = [("map_n", "int32", 1), ("final_n", "int32", 1), ("final_state", "float32", 132),
              ("counters", "int32", 30), ("n_entries", "int32", 1), ("status", "int32", 1),
              ("overflow", "int32", 1), ("llr_evals", "int32", 1)]


def _setup(n_rois, jumps):
    import torch
    from bamf_gb300 import rjstruct, synth
    b = synth.roi_batch_uneven(n_rois, seed=7)
    rj = rjstruct.uneven_rjstruct()
    rj.N_Burnin = rj.N_Trials = jumps
    dev = {k: torch.from_numpy(v).cuda() for k, v in
           (("data", b.data), ("offsets", b.offsets), ("xsize", b.xsize), ("ysize", b.ysize),
            ("psf_sigma", b.sigma))}
    return b, rj, dev


def _outs(n):
    import torch
    return {k: torch.full((n * w,), -7, dtype=getattr(torch, dt), device="cuda")
            for k, dt, w in OUT_FIELDS}


def _structs(dev, outs, n, side_max, bg0):
    from bamf_gb300 import sampler
    b = sampler.RoiBatch()
    b.n_rois = n
    b.side_max = side_max
    for k in ("data", "offsets", "xsize", "ysize", "psf_sigma"):
        setattr(b, k, dev[k].data_ptr())
    b.bg0 = bg0
    r = sampler.BatchResults()
    for k, t in outs.items():
        setattr(r, k, t.data_ptr())
    return b, r


def _host(outs):
    return {k: v.cpu().numpy() for k, v in outs.items()}


@pytest.mark.parametrize("arith,with_entries", [("fast", True), ("exact", True), ("fast", False)])
def test_noalloc_matches_workspace_entry_point_twice(cuda_lib, arith, with_entries):
    """Every per-ROI output equal, on two calls in a row.  Without an
    n_entries output the variant keeps the entry counts the MAP reduction
    needs in its own scratch section."""
    import torch
    from bamf_gb300 import abi, rjstruct, sampler
    L = sampler._declare()
    L.bamf_rjmcmc_batch_device_noalloc.restype = C.c_int
    L.bamf_rjmcmc_batch_device_noalloc.argtypes = [
        C.POINTER(sampler.RoiBatch), C.POINTER(abi.McmcParams), C.POINTER(sampler.Priors),
        C.c_uint32, C.c_int, C.POINTER(sampler.BatchResults), C.c_void_p]
    n, jumps = (240, 400) if arith == "fast" else (64, 150)
    b, rj, dev = _setup(n, jumps)
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    side_max = int(max(b.xsize.max(), b.ysize.max()))
    pr, keep = sampler.Sampler._priors(rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    mode = sampler.ARITH[arith]

    # existing entry point (workspace scratch)
    ref_outs = _outs(n)
    s = sampler.Sampler()
    s.run_device({**dev, "side_max": side_max}, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons,
                 seed=99, arith=arith, outs=ref_outs, bg0=bg0)
    torch.cuda.synchronize()
    ref = _host(ref_outs)
    assert (ref["status"] == 0).all()

    # the allocation-free variant, twice in a row on fresh output buffers
    for call in range(2):
        outs = _outs(n)
        if not with_entries:
            del outs["n_entries"]
        bs, rs = _structs(dev, outs, n, side_max, bg0)
        st = L.bamf_rjmcmc_batch_device_noalloc(C.byref(bs), C.byref(p), C.byref(pr), 99, mode,
                                                C.byref(rs), None)
        assert st == abi.BAMF_OK, (call, st)
        torch.cuda.synchronize()
        got = _host(outs)
        for k in got:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"call {call}: {k}")


def test_noalloc_rejects_batches_beyond_its_scratch(cuda_lib):
    from bamf_gb300 import abi, rjstruct, sampler
    L = sampler._declare()
    L.bamf_rjmcmc_batch_device_noalloc.restype = C.c_int
    L.bamf_rjmcmc_batch_device_noalloc.argtypes = [
        C.POINTER(sampler.RoiBatch), C.POINTER(abi.McmcParams), C.POINTER(sampler.Priors),
        C.c_uint32, C.c_int, C.POINTER(sampler.BatchResults), C.c_void_p]
    rj = rjstruct.uneven_rjstruct()  # 3000 + 3000 jumps: 6000 trace bytes per ROI
    p = rjstruct.mcmc_params(rj)
    pr, keep = sampler.Sampler._priors(rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    n = 10_000  # 60 MB of trace > BAMF_NOALLOC_SCRATCH_BYTES
    b = sampler.RoiBatch()
    b.n_rois = n
    b.side_max = 24
    dummy = np.zeros(16, np.int64)
    for k in ("data", "offsets", "xsize", "ysize"):
        setattr(b, k, dummy.ctypes.data)  # never dereferenced: rejected before any GPU work
    r = sampler.BatchResults()
    r.map_n = dummy.ctypes.data
    st = L.bamf_rjmcmc_batch_device_noalloc(C.byref(b), C.byref(p), C.byref(pr), 1, 1, C.byref(r), None)
    assert st == abi.BAMF_ERR_TOO_LARGE
