"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("bamf.h",):
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
