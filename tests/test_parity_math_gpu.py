"""The exact sampler's erf / log / exp (include/bamf_parity_math.h, double-
float arithmetic in single-precision operations) give the same bits on the
GPU as the same header compiled for the CPU, over the argument ranges the
sampler meets and the special values - the condition for the exact GPU
chains to equal the reference build's."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(fn, rng):
    if fn == 0:   # erf: stencil arguments (x - mu) / (sqrt 2 sigma)
        x = rng.uniform(-8.0, 8.0, 400_000)
        extra = [0.0, -0.0, 1e-30, -1e-30, 3.9999998, 4.0, -4.0, 1e-45, np.inf, -np.inf, np.nan]
    elif fn == 1:  # log: model ratios and counts, subnormal to huge
        x = np.exp(rng.uniform(-100.0, 88.0, 400_000))
        extra = [1e-45, 1.17549435e-38, 1.0, 2.0, 0.5, 3.4e38, 0.0, np.inf, -1.0, np.nan]
    else:          # exp: log-likelihood differences, normal and subnormal results
        x = rng.uniform(-106.0, 90.0, 400_000)
        extra = [0.0, -87.33655, -103.97, -104.0, 88.72, 89.0, -np.inf, np.inf, np.nan]
    return np.concatenate([x, extra]).astype(np.float32)


@pytest.mark.parametrize("fn,name", [(0, "erf"), (1, "log"), (2, "exp")])
def test_parity_math_device_equals_host(cuda_lib, oracle_port, fn, name):
    from bamf_gb300 import abi
    L = abi.lib()
    L.bamf_parity_math_device.restype = C.c_int
    L.bamf_parity_math_device.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    O = oracle_port.load("port")
    O.oracle_parity_math.restype = C.c_int
    O.oracle_parity_math.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    x = _inputs(fn, np.random.default_rng(fn))
    dev = np.zeros_like(x)
    host = np.zeros_like(x)
    assert L.bamf_parity_math_device(fn, x.ctypes.data, x.size, dev.ctypes.data) == 0
    assert O.oracle_parity_math(fn, x.ctypes.data, x.size, host.ctypes.data) == 0
    bad = np.flatnonzero(dev.view(np.uint32) != host.view(np.uint32))
    assert bad.size == 0, f"{name}: {bad.size} differ, first x={x[bad[0]]!r} gpu={dev[bad[0]]!r} cpu={host[bad[0]]!r}"
