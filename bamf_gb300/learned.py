"""Learned birth proposal over libbamf_gb300.so (include/bamf_cnn.h).

ProposalNet wraps the network handle: training on generator batches
(`train`), loss and gradient of a given batch (`loss_grad`), and inference
into the sampler's LEARNED birth tables (`infer`).  `generate` draws
synthetic 16x16 ROIs of the reference forward model on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

SIDE = 16
NPX = SIDE * SIDE
NPARAM = 28955
NCOUNT = 11
SYNTH_NMAX = 16


class SynthParams(C.Structure):
    _fields_ = [("mean_n", C.c_float), ("sigma", C.c_float), ("i_median", C.c_float),
                ("i_logsd", C.c_float), ("bg", C.c_float), ("bg_max", C.c_float)]


# the plain-RJMCMC generator (16x16, sigma 1.3, I ~ LogN(ln 1000, 0.3), bg 10)
# with Poisson(5) emitter counts: the training distribution of the network
C3_SYNTH = dict(mean_n=5.0, sigma=1.3, i_median=1000.0, i_logsd=0.3, bg=10.0, bg_max=0.0)


def _lib() -> C.CDLL:
    L = abi.lib()
    if getattr(L, "_cnn_declared", False):
        return L
    vp, i32, f32p = C.c_void_p, C.c_int, C.POINTER(C.c_float)
    L.bamf_synth_generate.argtypes = [C.POINTER(SynthParams), C.c_uint32, C.c_uint64, i32, vp, vp, vp, vp]
    L.bamf_cnn_create.argtypes = [C.POINTER(vp), C.c_uint32]
    L.bamf_cnn_destroy.argtypes = [vp]
    L.bamf_cnn_destroy.restype = None
    L.bamf_cnn_get_params.argtypes = [vp, f32p]
    L.bamf_cnn_set_params.argtypes = [vp, f32p]
    L.bamf_cnn_loss_grad.argtypes = [vp, vp, vp, vp, i32, f32p, f32p]
    L.bamf_cnn_train.argtypes = [vp, C.POINTER(SynthParams), i32, i32, C.c_float, C.c_uint32, f32p]
    L.bamf_cnn_train_examples.argtypes = [vp, vp, vp, vp, i32, i32, i32, C.c_float, f32p]
    L.bamf_cnn_infer.argtypes = [vp, vp, i32, vp, vp, vp, vp]
    L.bamf_cnn_init_states.argtypes = [vp, vp, vp, i32, C.c_float, i32, vp, vp, vp]
    for f in ("bamf_synth_generate", "bamf_cnn_create", "bamf_cnn_get_params", "bamf_cnn_set_params",
              "bamf_cnn_loss_grad", "bamf_cnn_train", "bamf_cnn_infer", "bamf_cnn_init_states"):
        getattr(L, f).restype = C.c_int
    L._cnn_declared = True
    return L


def _check(L, st, where):
    if st != abi.BAMF_OK:
        msg = L.bamf_last_error()
        raise abi.BamfError(st, f"{where} ({msg.decode() if msg else ''})")


def synth_params(**kw) -> SynthParams:
    d = dict(C3_SYNTH)
    d.update(kw)
    return SynthParams(**{k: float(v) for k, v in d.items()})


def generate(n: int, seed: int, first: int = 0, stream=None, **kw) -> dict:
    """n synthetic ROIs (torch CUDA tensors): data [n][256], n_em [n],
    xyi [n][16][3]."""
    import torch
    L = _lib()
    out = {"data": torch.empty((n, NPX), dtype=torch.float32, device="cuda"),
           "n_em": torch.empty(n, dtype=torch.int32, device="cuda"),
           "xyi": torch.empty((n, SYNTH_NMAX, 3), dtype=torch.float32, device="cuda")}
    sp = synth_params(**kw)
    st = L.bamf_synth_generate(C.byref(sp), int(seed), int(first), int(n), out["data"].data_ptr(),
                               out["n_em"].data_ptr(), out["xyi"].data_ptr(),
                               C.c_void_p(stream) if stream else None)
    _check(L, st, "bamf_synth_generate")
    return out


class ProposalNet:
    def __init__(self, seed: int = 0):
        L = _lib()
        h = C.c_void_p()
        _check(L, L.bamf_cnn_create(C.byref(h), int(seed)), "bamf_cnn_create")
        self._h, self._L = h, L

    def close(self):
        if self._h:
            self._L.bamf_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        p = np.zeros(NPARAM, np.float32)
        _check(self._L, self._L.bamf_cnn_get_params(self._h, abi.fptr(p)), "bamf_cnn_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != NPARAM:
            raise ValueError(f"expected {NPARAM} parameters")
        _check(self._L, self._L.bamf_cnn_set_params(self._h, abi.fptr(p)), "bamf_cnn_set_params")

    def loss_grad(self, batch: dict):
        """(loss, grad) of a batch dict from `generate` (torch CUDA tensors)."""
        n = int(batch["n_em"].numel())
        loss = np.zeros(1, np.float32)
        grad = np.zeros(NPARAM, np.float32)
        st = self._L.bamf_cnn_loss_grad(self._h, batch["data"].data_ptr(), batch["n_em"].data_ptr(),
                                        batch["xyi"].data_ptr(), n, abi.fptr(loss), abi.fptr(grad))
        _check(self._L, st, "bamf_cnn_loss_grad")
        return float(loss[0]), grad

    def train(self, steps: int, batch: int = 512, lr: float = 2e-3, data_seed: int = 1, **kw) -> np.ndarray:
        """Adam on fresh generator batches; returns the per-step batch loss."""
        sp = synth_params(**kw)
        trace = np.zeros(max(steps, 1), np.float32)
        st = self._L.bamf_cnn_train(self._h, C.byref(sp), int(steps), int(batch), float(lr), int(data_seed),
                                    abi.fptr(trace))
        _check(self._L, st, "bamf_cnn_train")
        return trace[:steps]

    def train_examples(self, ex: dict, steps: int, batch: int = 512, lr: float = 1e-3) -> np.ndarray:
        """Adam on caller examples (torch CUDA: data [n][256], n_em [n] int32,
        xyi [n][16][3]), e.g. from `examples_from_states`; per-step loss."""
        n = int(ex["n_em"].numel())
        trace = np.zeros(max(steps, 1), np.float32)
        st = self._L.bamf_cnn_train_examples(self._h, ex["data"].contiguous().data_ptr(),
                                             ex["n_em"].contiguous().data_ptr(), ex["xyi"].contiguous().data_ptr(),
                                             n, int(steps), int(batch), float(lr), abi.fptr(trace))
        _check(self._L, st, "bamf_cnn_train_examples")
        return trace[:steps]

    def infer(self, data, stream=None) -> dict:
        """data: torch CUDA float32 [n][256] (16x16 ROIs, y fastest) ->
        birth tables cdf [n*256], sub [n*256*16] and count logits [n][11]."""
        import torch
        n = int(data.shape[0])
        out = {"cdf": torch.empty(n * NPX, dtype=torch.float32, device="cuda"),
               "sub": torch.empty(n * NPX * 16, dtype=torch.float32, device="cuda"),
               "count_logits": torch.empty((n, NCOUNT), dtype=torch.float32, device="cuda")}
        st = self._L.bamf_cnn_infer(self._h, data.contiguous().data_ptr(), n, out["cdf"].data_ptr(),
                                    out["sub"].data_ptr(), out["count_logits"].data_ptr(),
                                    C.c_void_p(stream) if stream else None)
        _check(self._L, st, "bamf_cnn_infer")
        return out


def init_states(tables: dict, intensity: float = 1000.0, max_n: int = 10, stream=None) -> dict:
    """Sampler start states (init_n [n], init_ixy [n][3][32]) from `infer`'s
    output: argmax count, greedy most probable sub-cells."""
    import torch
    L = _lib()
    n = int(tables["count_logits"].shape[0])
    out = {"init_n": torch.zeros(n, dtype=torch.int32, device="cuda"),
           "init_ixy": torch.zeros((n, 3, 32), dtype=torch.float32, device="cuda")}
    st = L.bamf_cnn_init_states(tables["cdf"].data_ptr(), tables["sub"].data_ptr(),
                                tables["count_logits"].data_ptr(), n, float(intensity), int(max_n),
                                out["init_n"].data_ptr(), out["init_ixy"].data_ptr(),
                                C.c_void_p(stream) if stream else None)
    _check(L, st, "bamf_cnn_init_states")
    return out


def examples_from_states(data, pos_trace, n_entries, pos_thin: int, seed: int = 0) -> dict:
    """Training examples from states the sampler accepted: for every ROI one
    recorded state (bamf_batch_results.pos_trace) drawn uniformly from the
    second half of its chain (the trial phase when burn-in and trials are
    equally long), as targets: n_em = its Signal==1 count (clipped to
    BAMF_SYNTH_NMAX), xyi = the X, Y, I of those emitters.  data [n][256]
    are the ROIs the sampler ran on.  Torch CUDA in, torch CUDA out."""
    import torch
    n, pos_len, rec = pos_trace.shape
    S = (rec - 5) // 3
    ent = n_entries.to(torch.int64)
    nrec = torch.clamp((ent - 1) // pos_thin + 1, min=1, max=pos_len)
    lo = torch.minimum((ent // 2 + pos_thin - 1) // pos_thin, nrec - 1)
    g = torch.Generator(device=pos_trace.device)
    g.manual_seed(int(seed))
    u = torch.rand(n, generator=g, device=pos_trace.device)
    j = torch.minimum(lo + (u * (nrec - lo).to(torch.float32)).to(torch.int64), nrec - 1)
    r = pos_trace[torch.arange(n, device=pos_trace.device), j]
    ns = torch.nan_to_num(r[:, 1]).to(torch.int64).clamp(0, SYNTH_NMAX)
    k = torch.arange(SYNTH_NMAX, device=pos_trace.device)
    keep = (k[None, :] < ns[:, None]).to(torch.float32)
    xyi = torch.stack([r[:, 5:5 + SYNTH_NMAX], r[:, 5 + S:5 + S + SYNTH_NMAX],
                       r[:, 5 + 2 * S:5 + 2 * S + SYNTH_NMAX]], dim=2)
    xyi = torch.nan_to_num(xyi) * keep[:, :, None]
    return {"data": data.reshape(n, NPX).contiguous(), "n_em": ns.to(torch.int32).contiguous(),
            "xyi": xyi.contiguous()}
