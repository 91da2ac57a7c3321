"""The tcgen05 tensor-core path (TMEM allocation, MMA from shared-memory
descriptors, commit to an mbarrier, tcgen05.ld) on a known answer."""
import ctypes as C

import pytest

from bamf_gb300 import abi

pytestmark = pytest.mark.gpu


def test_tcgen05_mma_known_answer(cuda_lib):
    L = abi.lib()
    L.bamf_tcgen05_selftest.restype = C.c_int
    L.bamf_tcgen05_selftest.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_int)]
    err, to = C.c_double(), C.c_int()
    abi.check(L.bamf_tcgen05_selftest(C.byref(err), C.byref(to)), "bamf_tcgen05_selftest")
    print("tcgen05 128x32x16 bf16: max |error|", err.value, "timed out", to.value)
    assert to.value == 0
    assert err.value == 0.0


@pytest.mark.parametrize("layout", [0, 1], ids=["k_major", "mn_major"])
def test_tcgen05_mma_known_answer_per_layout(cuda_lib, layout):
    L = abi.lib()
    f = L.bamf_tcgen05_selftest_layout
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]
    err, to = C.c_double(), C.c_int()
    abi.check(f(layout, C.byref(err), C.byref(to)), "bamf_tcgen05_selftest_layout")
    assert to.value == 0
    assert err.value == 0.0
