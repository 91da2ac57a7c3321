"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("bamf.h", "bamf_cnn.h", "bamf_tiles.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]*?\b(bamf_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("bamf_crjmcmc_host", "bamf_rjmcmc_batch_device", "bamf_rjmcmc_batch_host",
              "bamf_workspace_create", "bamf_workspace_destroy", "bamf_version"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from bamf_gb300 import build
    path = build.build()
    import ctypes
    L = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    L.bamf_version.restype = ctypes.c_char_p
    assert b"sm_103a" in L.bamf_version()
    # never fails without a GPU
    assert L.bamf_device_count() >= 0


def test_host_entry_points_reject_bad_arguments_without_touching_the_gpu():
    import ctypes
    from bamf_gb300 import abi, build
    build.build()
    L = ctypes.CDLL(abi.LIB_PATH)
    L.bamf_crjmcmc_host.restype = ctypes.c_int
    # null data -> BAMF_ERR_INVALID_ARG before any CUDA call
    st = L.bamf_crjmcmc_host(None, 16, 16, None, None, None, 0, None, 0, None, 0, None, None, 0,
                             None, None, None, None, None)
    assert st == abi.BAMF_ERR_INVALID_ARG


def test_batch_proposal_and_trace_arguments_are_checked_before_the_gpu():
    """Non-reference proposals need fast arithmetic, LEARNED needs its
    tables, traces need a length (and one long enough for map_n)."""
    import ctypes as C

    import numpy as np

    from bamf_gb300 import abi, build, rjstruct, sampler
    build.build()
    L = sampler._declare()
    rj = rjstruct.c0_rjstruct()
    p = rjstruct.mcmc_params(rj)
    pr, keep = sampler.Sampler._priors(rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)
    data = np.zeros(256, np.float32)
    off = np.zeros(1, np.int64)
    side = np.full(1, 16, np.int32)
    out_i = np.zeros(1, np.int32)
    tr = np.zeros(8, np.uint8)

    def call(proposal=0, cdf=None, sub=None, arith=1, trace_len=0, n_trace=None, map_n=None):
        b = sampler.RoiBatch()
        b.n_rois = 1
        b.data, b.offsets, b.xsize, b.ysize = data.ctypes.data, off.ctypes.data, side.ctypes.data, side.ctypes.data
        b.proposal = proposal
        b.birth_cdf = cdf
        b.birth_sub = sub
        r = sampler.BatchResults()
        r.final_n = out_i.ctypes.data
        r.map_n = map_n
        r.trace_len = trace_len
        r.n_trace = n_trace
        ws = C.c_void_p()
        assert L.bamf_workspace_create(C.byref(ws)) == abi.BAMF_OK
        try:
            return L.bamf_rjmcmc_batch_host(ws, C.byref(b), C.byref(p), C.byref(pr), 1, arith, C.byref(r))
        finally:
            L.bamf_workspace_destroy(ws)

    assert call(proposal=1, arith=0) == abi.BAMF_ERR_INVALID_ARG        # uniform needs fast
    assert call(proposal=3) == abi.BAMF_ERR_INVALID_ARG                 # unknown proposal
    assert call(proposal=2) == abi.BAMF_ERR_INVALID_ARG                 # learned without tables
    assert call(n_trace=tr.ctypes.data) == abi.BAMF_ERR_INVALID_ARG     # trace without a length
    assert call(trace_len=8, n_trace=tr.ctypes.data, map_n=out_i.ctypes.data) == abi.BAMF_ERR_INVALID_ARG
    # well-formed calls get past the checks (and stop at the missing GPU here)
    ok = call(proposal=1, trace_len=8, n_trace=tr.ctypes.data)
    assert ok in (abi.BAMF_OK, abi.BAMF_ERR_NO_DEVICE)


def test_find_roi_pinned_rejects_bad_arguments_before_touching_the_device():
    """bamf_find_roi_pinned: no host frames or chunk_frames < 1 is
    BAMF_ERR_INVALID_ARG (checked on the host, no CUDA call); the Python
    wrapper rejects a host tensor of the wrong size."""
    import ctypes as C

    import numpy as np
    import torch

    from bamf_gb300 import abi, frontend
    fr = frontend.FindRoiDevice()
    L = fr._L
    buf = np.zeros(16, np.float32)
    out = np.zeros(3, np.int32)
    cnt = np.zeros(1, np.int64)
    common = (4, 4, 1, 1.3, 2.6, 7, 1.0, 1, out.ctypes.data, None, None, cnt.ctypes.data, None, None)
    assert L.bamf_find_roi_pinned(fr._ws, None, buf.ctypes.data, 8, *common) == abi.BAMF_ERR_INVALID_ARG
    assert L.bamf_find_roi_pinned(fr._ws, buf.ctypes.data, buf.ctypes.data, 0, *common) == \
        abi.BAMF_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        fr.run_pinned(torch.zeros(10), 4, 4, 1)
    fr.close()


def test_find_roi_fit_pinned_rejects_bad_arguments_before_touching_the_device():
    """bamf_find_roi_fit_pinned: missing crops or fit outputs, no capacity,
    a non-positive PSF sigma or negative iterations are
    BAMF_ERR_INVALID_ARG, a box beyond gaussMLE's 21 pixels
    BAMF_ERR_TOO_LARGE (checked on the host, no CUDA call)."""
    import numpy as np

    from bamf_gb300 import abi, frontend
    fr = frontend.FindRoiDevice()
    L = fr._L
    buf = np.zeros(16, np.float32)
    i32 = np.zeros(64, np.int32)
    f32 = np.zeros(64, np.float32)
    cnt = np.zeros(1, np.int64)

    def call(host=buf.ctypes.data, chunk=8, box=7, cap=4, psf=1.3, it=10, corners=i32.ctypes.data,
             stack=f32.ctypes.data, params=f32.ctypes.data, crlb=f32.ctypes.data, ll=f32.ctypes.data):
        return L.bamf_find_roi_fit_pinned(fr._ws, host, buf.ctypes.data, chunk, 4, 4, 1, 1.3, 2.6, box, 1.0, cap,
                                          psf, it, i32.ctypes.data, corners, stack, cnt.ctypes.data, params,
                                          crlb, ll, None)

    bad = abi.BAMF_ERR_INVALID_ARG
    assert call(host=None) == bad
    assert call(chunk=0) == bad
    assert call(cap=0) == bad
    assert call(psf=0.0) == bad
    assert call(it=-1) == bad
    assert call(corners=None) == bad
    assert call(stack=None) == bad
    assert call(params=None) == bad
    assert call(crlb=None) == bad
    assert call(ll=None) == bad
    assert call(box=22) == abi.BAMF_ERR_TOO_LARGE
    import torch
    with pytest.raises(ValueError):
        fr.run_fit_pinned(torch.zeros(10), 4, 4, 1)
    fr.close()


def test_crjmcmc_mirror_checks_the_model_option_on_the_host():
    """sampler.cRJMCMC (the MEX call, cRJMCMC.cpp:74): OptModel 0 or 1 only,
    and OptModel 1 needs a SampledPSF; both refused before any GPU call."""
    import numpy as np

    from bamf_gb300 import abi, sampler
    p = abi.McmcParams()
    E = {"N": 0, "I": [], "X": [], "Y": [], "BG": 10.0}
    pdf = np.ones(8, np.float32)
    with pytest.raises(abi.BamfError):
        sampler.cRJMCMC(np.zeros((8, 8), np.float32), E, p, 8, 8, pdf, pdf, pdf, OptModel=2)
    with pytest.raises(abi.BamfError):
        sampler.cRJMCMC(np.zeros((8, 8), np.float32), E, p, 8, 8, pdf, pdf, pdf, OptModel=1)
