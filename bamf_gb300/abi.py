"""ctypes mirror of include/bamf.h and the loader of libbamf_gb300.so.

The structs here are field-for-field copies of the C declarations; the
library itself is built in-tree by bamf_gb300/build.py.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbamf_gb300.so")

BAMF_OK = 0
BAMF_ERR_INVALID_ARG = 1
BAMF_ERR_CUDA = 2
BAMF_ERR_NO_DEVICE = 3
BAMF_ERR_TOO_LARGE = 4
BAMF_ERR_TIMEOUT = 5
BAMF_ERR_BAD_PRIOR = 6
BAMF_ERR_CAPACITY = 7
BAMF_ERR_UNSUPPORTED = 8
STATUS_NAMES = {
    0: "BAMF_OK", 1: "BAMF_ERR_INVALID_ARG", 2: "BAMF_ERR_CUDA", 3: "BAMF_ERR_NO_DEVICE",
    4: "BAMF_ERR_TOO_LARGE", 5: "BAMF_ERR_TIMEOUT", 6: "BAMF_ERR_BAD_PRIOR",
    7: "BAMF_ERR_CAPACITY", 8: "BAMF_ERR_UNSUPPORTED",
}

BAMF_NMAX = 32
BAMF_MAX_ROI_SIDE = 32
BAMF_ARITH_EXACT = 0
BAMF_ARITH_FAST = 1


class BamfError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where} failed: {STATUS_NAMES.get(status, status)}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != BAMF_OK:
        raise BamfError(status, where)


class McmcParams(C.Structure):
    """bamf_mcmc_params: the MATLAB `MCMC` struct (rjmcmc.m:49-78)."""
    _fields_ = [
        ("PSFsigma", C.c_float),
        ("N_Trials", C.c_int32),
        ("N_Burnin", C.c_int32),
        ("I_stdFg", C.c_float), ("I_stdBg", C.c_float),
        ("X_stdFg", C.c_float), ("X_stdBg", C.c_float),
        ("P_Burnin", C.c_float * 8),
        ("P_Trials", C.c_float * 8),
        ("Rho", C.c_float),
        ("Bnd_out", C.c_float),
        ("Grid_Zoom", C.c_int32),
        ("Split_std", C.c_float),
        ("Icutoff", C.c_float),
        ("BG_std", C.c_float),
        ("ABBG_std", C.c_float),
        ("DX", C.c_float),
        ("DriftX", C.c_float), ("DriftY", C.c_float),
        ("PSFsize", C.c_int32 * 4),
        ("IsBackg", C.c_int32),
    ]


class Emitters(C.Structure):
    _fields_ = [
        ("N", C.c_int32),
        ("I", C.POINTER(C.c_float)),
        ("X", C.POINTER(C.c_float)),
        ("Y", C.POINTER(C.c_float)),
        ("BG", C.c_float),
    ]


class Rng(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("chain_id", C.c_uint32), ("offset", C.c_uint32)]


class Chain(C.Structure):
    _fields_ = [
        ("capacity_entries", C.c_int32),
        ("capacity_records", C.c_int32),
        ("n_entries", C.c_int32),
        ("n_records", C.c_int32),
        ("N", C.POINTER(C.c_int32)),
        ("LLR", C.POINTER(C.c_float)),
        ("PR", C.POINTER(C.c_float)),
        ("JumpType", C.POINTER(C.c_int32)),
        ("Accepted", C.POINTER(C.c_int32)),
        ("BG", C.POINTER(C.c_float)),
        ("ABG", C.POINTER(C.c_float)),
        ("BBG", C.POINTER(C.c_float)),
        ("Index", C.POINTER(C.c_int32)),
        ("Photons", C.POINTER(C.c_float)),
        ("X", C.POINTER(C.c_float)),
        ("Y", C.POINTER(C.c_float)),
        ("Signal", C.POINTER(C.c_int32)),
    ]


COUNTER_NAMES = [
    "N_jump", "N_split", "N_merge", "N_birth", "N_death",
    "A_jump", "A_split", "A_merge", "A_birth", "A_death",
    "N_jumpFg", "N_splitFg", "N_mergeFg", "N_birthFg", "N_deathFg",
    "A_jumpFg", "A_splitFg", "A_mergeFg", "A_birthFg", "A_deathFg",
    "N_jumpBg", "N_splitBg", "N_mergeBg", "N_birthBg", "N_deathBg",
    "A_jumpBg", "A_splitBg", "A_mergeBg", "A_birthBg", "A_deathBg",
]


class Counters(C.Structure):
    _fields_ = [(n, C.c_int32) for n in COUNTER_NAMES]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n in COUNTER_NAMES}


ENTRY_FIELDS = [("N", np.int32), ("LLR", np.float32), ("PR", np.float32),
                ("JumpType", np.int32), ("Accepted", np.int32), ("BG", np.float32),
                ("ABG", np.float32), ("BBG", np.float32)]
RECORD_FIELDS = [("Index", np.int32), ("Photons", np.float32), ("X", np.float32),
                 ("Y", np.float32), ("Signal", np.int32)]


def alloc_chain(cap_entries: int, cap_records: int):
    """A bamf_chain whose arrays are numpy buffers; returns (struct, arrays)."""
    arrays = {}
    ch = Chain()
    ch.capacity_entries = cap_entries
    ch.capacity_records = cap_records
    for name, dt in ENTRY_FIELDS:
        a = np.zeros(max(cap_entries, 1), dtype=dt)
        arrays[name] = a
        ctype = C.c_int32 if dt == np.int32 else C.c_float
        setattr(ch, name, a.ctypes.data_as(C.POINTER(ctype)))
    for name, dt in RECORD_FIELDS:
        a = np.zeros(max(cap_records, 1), dtype=dt)
        arrays[name] = a
        ctype = C.c_int32 if dt == np.int32 else C.c_float
        setattr(ch, name, a.ctypes.data_as(C.POINTER(ctype)))
    return ch, arrays


def chain_to_dict(ch: Chain, arrays: dict) -> dict:
    out = {}
    for name, _ in ENTRY_FIELDS:
        out[name] = arrays[name][: ch.n_entries].copy()
    for name, _ in RECORD_FIELDS:
        out[name] = arrays[name][: ch.n_records].copy()
    return out


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def make_emitters(n: int, I=None, X=None, Y=None, BG: float = 0.0):
    """bamf_emitters plus the numpy buffers that must outlive it."""
    keep = []
    e = Emitters()
    e.N = int(n)
    e.BG = float(BG)
    for name, arr in (("I", I), ("X", X), ("Y", Y)):
        if n > 0:
            a = np.ascontiguousarray(arr, dtype=np.float32)
            keep.append(a)
            setattr(e, name, fptr(a))
        else:
            setattr(e, name, C.POINTER(C.c_float)())
    return e, keep


_lib = None


def lib() -> C.CDLL:
    """The in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            )
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L: C.CDLL) -> None:
    vp = C.c_void_p
    i32 = C.c_int32
    f32 = C.c_float
    pf = C.POINTER(C.c_float)
    pi = C.POINTER(C.c_int32)
    L.bamf_version.restype = C.c_char_p
    L.bamf_device_count.restype = C.c_int
    L.bamf_crjmcmc_host.restype = C.c_int
    L.bamf_crjmcmc_host.argtypes = [
        pf, C.c_int, C.c_int, C.POINTER(Emitters), C.POINTER(McmcParams),
        pf, C.c_int, pf, C.c_int, pf, C.c_int, pf, C.POINTER(Rng), C.c_int,
        pf, pf, C.POINTER(Chain), C.POINTER(Chain), C.POINTER(Counters),
    ]
    del vp, i32, f32, pi
