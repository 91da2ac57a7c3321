"""TEST INFRASTRUCTURE: Python access to the CPU oracles.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, and only as the checker (or the timed CPU baseline); the
product never imports it.

Libraries (built by oracle/Makefile):
  port         _build/liboracle.so          project C restatement, parity math
  port_native  _build/liboracle_native.so   same, glibc float math
  ref          _ref/libref_rjmcmc.so        the reference sampler, parity math
  ref_native   _ref/libref_rjmcmc_native.so the reference sampler, glibc math
The `ref` variants exist only where the reference tree could be compiled.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from bamf_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
# where the reference sampler sources are staged for machines without the
# reference tree (git-ignored; `make -C oracle stage-ref`)
STAGED_REF = os.path.join(HERE, "_ref", "src")
PATHS = {
    "port": os.path.join(HERE, "_build", "liboracle.so"),
    "port_native": os.path.join(HERE, "_build", "liboracle_native.so"),
    "ref": os.path.join(HERE, "_ref", "libref_rjmcmc.so"),
    "ref_native": os.path.join(HERE, "_ref", "libref_rjmcmc_native.so"),
}
PREFIX = {"port": "oracle", "port_native": "oracle", "ref": "ref", "ref_native": "ref"}
_libs: dict = {}


def _has_sampler_sources(d: str | None) -> bool:
    return bool(d) and os.path.isfile(os.path.join(d, "source", "c", "LibRJMCMC.cpp"))


def ref_dir() -> str | None:
    """The reference tree named by $BAMF_REFERENCE_DIR, else the staged copy
    of its sampler sources, else None."""
    d = os.environ.get("BAMF_REFERENCE_DIR")
    if _has_sampler_sources(d):
        return d
    return STAGED_REF if _has_sampler_sources(STAGED_REF) else None


def build(ref: bool | None = None) -> None:
    """Compile the port (always) and the reference sampler oracle (when its
    sources can be found; with the full reference tree also stage them for
    machines that lack it)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    d = ref_dir()
    if d and d != STAGED_REF:
        subprocess.run(["make", "-s", "-C", HERE, "stage-ref", f"REF_DIR={d}"], check=True)
        # the reference's CUDA front-end kernels as sm_103a cubins (nvcc
        # cross-compiles them here; the cubins travel to the GPU host)
        subprocess.run(["make", "-s", "-C", HERE, "ref-cubin", f"REF_DIR={d}"], check=True)
    if ref is None:
        ref = d is not None
    if ref:
        if d is None:
            raise FileNotFoundError("reference sampler sources not found: set BAMF_REFERENCE_DIR")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={d}"], check=True)


def available(kind: str) -> bool:
    return os.path.exists(PATHS[kind])


def load(kind: str = "port") -> C.CDLL:
    if kind in _libs:
        return _libs[kind]
    if not os.path.exists(PATHS[kind]):
        if kind.startswith("port"):
            build(ref=False)
        else:
            raise FileNotFoundError(f"{PATHS[kind]} not built (reference sources unavailable)")
    L = C.CDLL(PATHS[kind])
    p = PREFIX[kind]
    pf = C.POINTER(C.c_float)
    run = getattr(L, f"{p}_rjmcmc_run")
    run.restype = C.c_void_p
    run.argtypes = [pf, C.c_int, C.c_int, C.POINTER(abi.Emitters), C.POINTER(abi.McmcParams),
                    pf, C.c_int, pf, C.c_int, pf, C.c_int, pf, C.POINTER(abi.Rng)]
    run_m = getattr(L, f"{p}_rjmcmc_run_model")
    run_m.restype = C.c_void_p
    run_m.argtypes = [pf, C.c_int, C.c_int, C.POINTER(abi.Emitters), C.POINTER(abi.McmcParams),
                      pf, C.c_int, pf, C.c_int, pf, C.c_int, pf, pf, C.c_int, C.POINTER(abi.Rng)]
    getattr(L, f"{p}_result_sizes").argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    getattr(L, f"{p}_result_chain").argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.Chain)]
    getattr(L, f"{p}_result_grids").argtypes = [C.c_void_p, pf, pf]
    getattr(L, f"{p}_result_counters").argtypes = [C.c_void_p, C.POINTER(abi.Counters)]
    getattr(L, f"{p}_result_free").argtypes = [C.c_void_p]
    pi = C.POINTER(C.c_int32)
    getattr(L, f"{p}_rjmcmc_batch").argtypes = [
        pf, C.POINTER(C.c_int64), pi, pi, pf, C.c_int, C.POINTER(abi.McmcParams),
        pf, C.c_int, pf, C.c_int, pf, C.c_int, C.c_float, C.c_uint32, C.c_int, pi, pi, pi]
    if kind.startswith("port"):
        L.oracle_findroi_filter.argtypes = [pf, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                            C.c_int, C.c_float, pf, C.c_int]
        L.oracle_findroi_dog.argtypes = [pf, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, pf]
        L.oracle_gaussmle_xynb.argtypes = [pf, C.c_int, C.c_int, C.c_float, C.c_int, pf, pf, pf,
                                           C.c_int]
        pd = C.POINTER(C.c_double)
        L.oracle_gaussmle_xynb_f64.argtypes = [pf, C.c_int, C.c_int, C.c_double, C.c_int, pd, pd,
                                               pd, C.c_int]
    _libs[kind] = L
    return L


def run_chain(kind: str, roi: np.ndarray, params: abi.McmcParams, off: np.ndarray,
              sig: np.ndarray, back: np.ndarray, e0=None, rng=(0, 0, 0),
              scmos: np.ndarray | None = None, sampled_psf: np.ndarray | None = None) -> dict:
    """One cRJMCMC run on a (Ysize, Xsize) ROI; returns the raw outputs.

    e0 = (I, X, Y, BG) or None for the empty start of rjmcmc.m (BG taken
    from the offset prior's maximum by the caller); sampled_psf, a 4-D array
    of shape params.PSFsize, selects OptModel 1."""
    L = load(kind)
    p = PREFIX[kind]
    ysize, xsize = roi.shape
    data = np.ascontiguousarray(roi.ravel(order="F"), dtype=np.float32)
    if e0 is None:
        e0 = ([], [], [], 0.0)
    I, X, Y, BG = e0
    em, keep = abi.make_emitters(len(I), I, X, Y, BG)
    off = np.ascontiguousarray(off, np.float32)
    sig = np.ascontiguousarray(sig, np.float32)
    back = np.ascontiguousarray(back, np.float32)
    sc = None if scmos is None else np.ascontiguousarray(np.asarray(scmos).ravel(order="F"),
                                                         np.float32)
    r = abi.Rng(*rng)
    psf = None
    if sampled_psf is not None:
        if tuple(params.PSFsize) != tuple(np.shape(sampled_psf)):
            raise ValueError("params.PSFsize must be the sampled PSF's shape")
        psf = np.ascontiguousarray(np.asarray(sampled_psf, np.float32).ravel(order="F"))
    h = getattr(L, f"{p}_rjmcmc_run_model")(abi.fptr(data), xsize, ysize, C.byref(em), C.byref(params),
                                            abi.fptr(off), off.size, abi.fptr(sig), sig.size,
                                            abi.fptr(back), back.size,
                                            abi.fptr(sc) if sc is not None else None,
                                            abi.fptr(psf) if psf is not None else None,
                                            1 if psf is not None else 0, C.byref(r))
    if not h:
        raise ValueError("oracle rejected the arguments")
    try:
        sizes = (C.c_int64 * 7)()
        getattr(L, f"{p}_result_sizes")(h, sizes)
        out = {"uniforms_used": int(sizes[5]), "messages": int(sizes[6])}
        for w, name in ((0, "chain"), (1, "chain_test")):
            ne, nr = int(sizes[2 * w]), int(sizes[2 * w + 1])
            ch, arrs = abi.alloc_chain(ne, nr)
            abi.check(getattr(L, f"{p}_result_chain")(h, w, C.byref(ch)), "result_chain")
            out[name] = abi.chain_to_dict(ch, arrs)
        g = int(sizes[4])
        pg = np.zeros(g, np.float32)
        pb = np.zeros(g, np.float32)
        getattr(L, f"{p}_result_grids")(h, abi.fptr(pg), abi.fptr(pb))
        Z = params.Grid_Zoom
        out["pgrid"] = pg.reshape(xsize * Z, ysize * Z).T.copy()
        out["pback"] = pb.reshape(xsize * Z, ysize * Z).T.copy()
        c = abi.Counters()
        getattr(L, f"{p}_result_counters")(h, C.byref(c))
        out["counters"] = c.as_dict()
    finally:
        getattr(L, f"{p}_result_free")(h)
    return out


def run_batch(batch, params: abi.McmcParams, off, sig, back, bg0: float, seed: int,
              threads: int = 1, kind: str = "port_native") -> dict:
    """Per-ROI summaries (final N, MAP N, accepted moves) on host threads;
    kind "port"/"port_native" (the restatement) or "ref"/"ref_native" (the
    reference sampler build)."""
    L = load(kind)
    batch_fn = getattr(L, f"{PREFIX[kind]}_rjmcmc_batch")
    n = batch.n
    fn = np.zeros(n, np.int32)
    mn = np.zeros(n, np.int32)
    na = np.zeros(n, np.int32)
    off = np.ascontiguousarray(off, np.float32)
    sig = np.ascontiguousarray(sig, np.float32)
    back = np.ascontiguousarray(back, np.float32)
    pi = C.POINTER(C.c_int32)
    abi.check(batch_fn(
        abi.fptr(batch.data), batch.offsets.ctypes.data_as(C.POINTER(C.c_int64)),
        batch.xsize.ctypes.data_as(pi), batch.ysize.ctypes.data_as(pi),
        abi.fptr(np.ascontiguousarray(batch.sigma, np.float32)), n, C.byref(params),
        abi.fptr(off), off.size, abi.fptr(sig), sig.size, abi.fptr(back), back.size,
        float(bg0), int(seed), int(threads), fn.ctypes.data_as(pi), mn.ctypes.data_as(pi),
        na.ctypes.data_as(pi)), "oracle_rjmcmc_batch")
    return {"final_n": fn, "map_n": mn, "n_accepted": na}


def findroi_dog(stack: np.ndarray, sigma1: float = 1.3, sigma2: float = 2.6) -> np.ndarray:
    """The difference-of-Gaussians image of findROI's kernels (gaussX /
    gaussY per sigma, subtract) for a (Y, X, Z) stack; returned flat in the
    stack's memory order (y fastest)."""
    L = load("port")
    st = np.asarray(stack, np.float32)
    if st.ndim == 2:
        st = st[:, :, None]
    ys, xs, zs = st.shape
    flat = np.ascontiguousarray(st.ravel(order="F"))
    dog = np.zeros_like(flat)
    abi.check(L.oracle_findroi_dog(abi.fptr(flat), ys, xs, zs, float(sigma1), float(sigma2), abi.fptr(dog)),
              "oracle_findroi_dog")
    return dog


def findroi(stack: np.ndarray, sigma1: float = 1.3, sigma2: float = 2.6, boxsize: int = 7,
            minval: float | None = None, threads: int = 8) -> dict:
    """findROI.m restated: flags from the kernels' restatement, then find /
    ind2sub (:125-126), the box clamp (:130-148) and the crop (:157-163)."""
    import math
    L = load("port")
    st = np.asarray(stack, np.float32)
    if st.ndim == 2:
        st = st[:, :, None]
    ys, xs, zs = st.shape
    flat = np.ascontiguousarray(st.ravel(order="F"))
    flags = np.zeros(flat.size, np.float32)
    if minval is None:
        minval = (1 / 4) * 2000 * (1 / (2 * math.pi * 2 * 1.3 ** 2))
    abi.check(L.oracle_findroi_filter(abi.fptr(flat), ys, xs, zs, float(sigma1), float(sigma2),
                                      int(boxsize), float(np.float32(minval)), abi.fptr(flags),
                                      int(threads)), "oracle_findroi_filter")
    m = np.flatnonzero(flags)
    Ii = m % ys + 1
    Jj = (m // ys) % xs + 1
    Kk = m // (ys * xs) + 1
    half = int(np.floor(boxsize / 2 + 0.5))
    sr = Ii - half + 1
    mr = sr < 1
    sr[mr] = 1
    sc = Jj - half + 1
    mc = sc < 1
    sc[mc] = 1
    er = sr + boxsize - 1
    er[mr] = boxsize
    lr = er > ys
    er[lr] = ys
    sr[lr] = ys - boxsize + 1
    ec = sc + boxsize - 1
    ec[mc] = boxsize
    lc = ec > xs
    ec[lc] = xs
    sc[lc] = xs - boxsize + 1
    rois = np.zeros((boxsize, boxsize, len(m)), np.float32)
    for b in range(len(m)):
        rois[:, :, b] = st[sr[b] - 1:er[b], sc[b] - 1:ec[b], Kk[b] - 1]
    return {"coords": np.stack([Ii, Jj, Kk], 1).astype(np.int32), "YBoxCorner": sr.astype(np.int32),
            "XBoxCorner": sc.astype(np.int32), "ROIStack": rois, "flags": flags}


def gaussmle(rois: np.ndarray, sigma: float, iterations: int, double: bool = False,
             threads: int = 8) -> dict:
    """kernel_MLEFit_XYNB_ restated (float, or double as the FP64 oracle);
    rois (sz, sz, N); outputs param-major like the kernel."""
    L = load("port")
    d = np.ascontiguousarray(np.asarray(rois, np.float32).ravel(order="F"))
    sz, _, n = np.asarray(rois).shape
    if double:
        dt, fn = np.float64, L.oracle_gaussmle_xynb_f64
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    else:
        dt, fn = np.float32, L.oracle_gaussmle_xynb
        ptr = abi.fptr
    P = np.zeros(4 * n, dt)
    CR = np.zeros(4 * n, dt)
    LLv = np.zeros(n, dt)
    abi.check(fn(abi.fptr(d), sz, n, sigma, int(iterations), ptr(P), ptr(CR), ptr(LLv), int(threads)),
              "oracle_gaussmle")
    return {"P": P.reshape(4, n).T, "CRLB": CR.reshape(4, n).T, "LL": LLv}
