"""Builds bamf_gb300/libbamf_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel; the sampler's exact
instantiation is compiled with -fmad=false so that nvcc fuses no float
multiply-add (its chain must round like the reference's), the fast one with
-use_fast_math.  Rebuilds only
when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "libbamf_gb300.so")
OBJDIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]
# The exact sampler must round every float operation as the reference does;
# the fast sampler promises no bitwise parity, and approximate division and
# square root shrink its code (the chain loop is instruction-cache bound).
PER_FILE = {"sampler_exact.cu": ["-fmad=false"], "sampler_exact_num.cu": ["-fmad=false"],
            "sampler_fast.cu": ["-use_fast_math"], "sampler_fast_num.cu": ["-use_fast_math"]}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__]
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj] + COMMON + PER_FILE.get(os.path.basename(src), []) + extra
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build_boundary() -> None:
    """The MEX gateways (mex/, against the project's mx stub) and the
    standalone C++ driver (driver/), both linking the library."""
    for d in ("mex", "driver"):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, d)], check=True)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile every .cu under csrc/ and link the shared library, then the
    MEX gateways and the driver that link it; returns the library's path."""
    if not force and not _stale():
        build_boundary()
        return OUT
    os.makedirs(OBJDIR, exist_ok=True)
    extra = extra or []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose), sources()))
    tmp = OUT + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + ARCH + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    build_boundary()
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
    print(OUT)
