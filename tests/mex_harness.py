"""Calls the MEX gateways of mex/ from Python the way MATLAB would, through
the project's mx stub (mex/stub): numpy arrays, numbers, strings and dicts
become mxArrays (column-major, MATLAB classes), the gateway's outputs come
back as numpy arrays and dicts (struct arrays as lists of dicts)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CLASS = {np.dtype(np.float64): 6, np.dtype(np.float32): 7, np.dtype(np.int8): 8, np.dtype(np.uint8): 9,
         np.dtype(np.int16): 10, np.dtype(np.uint16): 11, np.dtype(np.int32): 12, np.dtype(np.uint32): 13,
         np.dtype(np.int64): 14, np.dtype(np.uint64): 15}
DTYPE = {v: k for k, v in CLASS.items()}
STRUCT, CHAR = 2, 4


class MexError(Exception):
    def __init__(self, ident: str, msg: str):
        super().__init__(f"{ident}: {msg}")
        self.ident = ident


def build() -> None:
    """Builds the library, then the gateways and the driver (make)."""
    from bamf_gb300 import build as b
    b.build()


class Gateway:
    def __init__(self, name: str):
        build()
        self.L = L = C.CDLL(os.path.join(ROOT, "mex", "_build", f"{name}.so"))
        vp, sz = C.c_void_p, C.c_size_t
        L.mxCreateNumericArray.restype = vp
        L.mxCreateNumericArray.argtypes = [sz, C.POINTER(sz), C.c_int, C.c_int]
        L.mxCreateStructMatrix.restype = vp
        L.mxCreateStructMatrix.argtypes = [sz, sz, C.c_int, C.POINTER(C.c_char_p)]
        L.mxCreateString.restype = vp
        L.mxCreateString.argtypes = [C.c_char_p]
        L.mxSetField.argtypes = [vp, sz, C.c_char_p, vp]
        L.mxGetData.restype = vp
        L.mxGetData.argtypes = [vp]
        L.mxGetClassID.argtypes = [vp]
        L.mxGetNumberOfDimensions.restype = sz
        L.mxGetNumberOfDimensions.argtypes = [vp]
        L.mxGetDimensions.restype = C.POINTER(sz)
        L.mxGetDimensions.argtypes = [vp]
        L.mxGetNumberOfElements.restype = sz
        L.mxGetNumberOfElements.argtypes = [vp]
        L.mxGetNumberOfFields.argtypes = [vp]
        L.mxGetFieldNameByNumber.restype = C.c_char_p
        L.mxGetFieldNameByNumber.argtypes = [vp, C.c_int]
        L.mxGetFieldByNumber.restype = vp
        L.mxGetFieldByNumber.argtypes = [vp, sz, C.c_int]
        L.mxGetString.argtypes = [vp, C.c_char_p, sz]
        L.mxDestroyArray.argtypes = [vp]
        L.mx_stub_call_gateway.argtypes = [C.c_int, C.POINTER(vp), C.c_int, C.POINTER(vp), C.c_char_p, sz,
                                           C.c_char_p, sz]

    # ---------------------------------------------------------------- to MATLAB
    def to_mx(self, v):
        L = self.L
        if isinstance(v, dict):
            names = list(v)
            arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
            s = L.mxCreateStructMatrix(1, 1, len(names), arr)
            for n in names:
                L.mxSetField(s, 0, n.encode(), self.to_mx(v[n]))
            return s
        if isinstance(v, str):
            return L.mxCreateString(v.encode())
        a = np.asarray(v)
        if a.dtype == np.float16 or a.dtype.kind == "b":
            a = a.astype(np.float64)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        elif a.ndim == 1:
            a = a.reshape(1, -1)
        dims = (C.c_size_t * a.ndim)(*a.shape)
        m = L.mxCreateNumericArray(a.ndim, dims, CLASS[a.dtype], 0)
        flat = np.ascontiguousarray(a.ravel(order="F"))
        if flat.nbytes:
            C.memmove(L.mxGetData(m), flat.ctypes.data, flat.nbytes)
        return m

    # -------------------------------------------------------------- from MATLAB
    def from_mx(self, m):
        L = self.L
        if not m:
            return None
        cls = L.mxGetClassID(m)
        nd = L.mxGetNumberOfDimensions(m)
        dims = tuple(L.mxGetDimensions(m)[k] for k in range(nd))
        if cls == STRUCT:
            nf = L.mxGetNumberOfFields(m)
            names = [L.mxGetFieldNameByNumber(m, f).decode() for f in range(nf)]
            out = [{n: self.from_mx(L.mxGetFieldByNumber(m, i, f)) for f, n in enumerate(names)}
                   for i in range(int(np.prod(dims)))]
            return out[0] if len(out) == 1 and dims == (1, 1) else out
        if cls == CHAR:
            buf = C.create_string_buffer(int(np.prod(dims)) + 1)
            L.mxGetString(m, buf, len(buf))
            return buf.value.decode()
        dt = DTYPE[cls]
        n = int(np.prod(dims))
        a = np.empty(n, dt)
        if n:
            C.memmove(a.ctypes.data, L.mxGetData(m), a.nbytes)
        return a.reshape(dims, order="F")

    def __call__(self, nlhs: int, *args):
        """Calls mexFunction(nlhs, plhs, nrhs, prhs); returns the nlhs
        outputs (converted), or raises MexError with the gateway's
        identifier."""
        L = self.L
        prhs = (C.c_void_p * max(len(args), 1))(*[self.to_mx(a) for a in args])
        plhs = (C.c_void_p * max(nlhs, 1))()
        eid = C.create_string_buffer(256)
        emsg = C.create_string_buffer(1024)
        try:
            rc = L.mx_stub_call_gateway(nlhs, plhs, len(args), prhs, eid, len(eid), emsg, len(emsg))
            if rc:
                raise MexError(eid.value.decode(), emsg.value.decode())
            return [self.from_mx(plhs[k]) for k in range(max(nlhs, 1) if plhs[0] else 0)][:max(nlhs, 1)]
        finally:
            for k in range(len(args)):
                L.mxDestroyArray(prhs[k])
            for k in range(max(nlhs, 1)):
                if plhs[k]:
                    L.mxDestroyArray(plhs[k])


def driver_path() -> str:
    build()
    return os.path.join(ROOT, "driver", "_build", "bamf_driver")


def run_driver(*args, check=True):
    return subprocess.run([driver_path(), *map(str, args)], capture_output=True, text=True, check=check)
