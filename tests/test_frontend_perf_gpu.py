"""Front-end speed against the reference's own kernels on the same GPU.

FindROI on the 2000-frame 256x256 stack and gaussMLE (7x7, 10 iterations)
on the maxima it finds: this implementation's device calls against the
reference's FindROI / gaussMLE kernels (compiled unmodified for sm_103a,
oracle/refgpu.py) launched with the reference geometry.  The reference time
counts kernel execution only (its MATLAB glue also copies every
intermediate back to the host, findROI.m:189-222, which is left out in its
favour).  Prints the timings; asserts this implementation is not slower."""
import ctypes as C

import numpy as np
import pytest

from bamf_gb300 import frontend, synth

pytestmark = pytest.mark.gpu


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def test_frontend_not_slower_than_the_reference_kernels(cuda_lib):
    import torch

    from oracle import refgpu
    if not (refgpu.available("findroi") and refgpu.available("gaussmle")):
        pytest.skip("reference cubins not built (make -C oracle ref-cubin)")
    Z = 2000
    stack, _ = synth.frames(Z, seed=3)
    dev = torch.from_numpy(np.asfortranarray(stack).ravel(order="F")).cuda()
    n = dev.numel()
    mv = frontend.default_minval()
    fr = frontend.FindRoiDevice()
    for _ in range(2):
        out = fr.run(dev, 256, 256, Z, boxsize=7, minval=mv)
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        e0, e1 = _events()
        e0.record()
        out = fr.run(dev, 256, 256, Z, boxsize=7, minval=mv)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ours_findroi = min(ts)
    count = int(out["count"].item())

    # reference kernels, kernel time only
    d = refgpu.driver()
    ptr = lambda t: C.c_uint64(t.data_ptr())  # noqa: E731
    bufs = {k: torch.empty(n, dtype=torch.float32, device="cuda") for k in ("a", "b")}
    sub = torch.full((n + 1024,), float("nan"), dtype=torch.float32, device="cuda")
    im1 = torch.empty(n, dtype=torch.float32, device="cuda")
    res = torch.empty(n, dtype=torch.float32, device="cuda")
    ref_ms = 0.0

    def timed(which, name, grid, block, args):
        nonlocal ref_ms
        e0, e1 = _events()
        e0.record()
        d.launch(which, name, grid, block, args)
        e1.record()
        torch.cuda.synchronize()
        ref_ms += e0.elapsed_time(e1)

    for rep in range(2):
        ref_ms = 0.0
        for key, sg in (("a", 1.3), ("b", 2.6)):
            bufs[key].copy_(dev)
            cf = refgpu._coeffs(sg)
            timed("findroi", "gaussX", (Z,), (256,), [ptr(bufs[key]), C.c_int(256)] + cf)
            timed("findroi", "gaussY", (Z,), (256,), [ptr(bufs[key]), C.c_int(256)] + cf)
        sub[:n].copy_(bufs["a"])
        timed("findroi", "subtract", (256, Z), (256,), [ptr(sub), ptr(bufs["b"])])
        im1.copy_(bufs["a"])
        timed("findroi", "maxX", (256, Z), (256,), [ptr(sub), ptr(im1), C.c_int(7), C.c_float(mv)])
        res.copy_(sub[:n])
        timed("findroi", "maxY", (256, Z), (256,), [ptr(res), ptr(im1), C.c_int(7), C.c_float(mv)])
    ref_findroi = ref_ms

    rois = out["stack"][:count].contiguous()
    for _ in range(2):
        frontend.gauss_mle_device(rois, 7, count, 1.3, 10)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    frontend.gauss_mle_device(rois, 7, count, 1.3, 10)
    e1.record()
    torch.cuda.synchronize()
    ours_mle = e0.elapsed_time(e1)
    P = torch.zeros(4 * count, dtype=torch.float32, device="cuda")
    CR = torch.zeros_like(P)
    LL = torch.zeros(count, dtype=torch.float32, device="cuda")
    args = [ptr(rois), C.c_float(1.3), C.c_int(7), C.c_int(10), ptr(P), ptr(CR), ptr(LL), C.c_int(count)]
    for _ in range(2):
        d.launch("gaussmle", "mle_xynb", ((count + 127) // 128,), (128,), args)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    d.launch("gaussmle", "mle_xynb", ((count + 127) // 128,), (128,), args)
    e1.record()
    torch.cuda.synchronize()
    ref_mle = e0.elapsed_time(e1)
    gbs = 4.0 * n / (ours_findroi * 1e-3) / 1e9
    print(f"\nFindROI 2000x256x256: this {ours_findroi:.2f} ms ({Z / ours_findroi * 1e3:.0f} frames/s, "
          f"{gbs:.0f} GB/s of one 4-byte read per pixel), reference kernels {ref_findroi:.2f} ms "
          f"({ref_findroi / ours_findroi:.2f}x); maxima {count}")
    print(f"gaussMLE 7x7 x {count}, 10 iterations: this {ours_mle:.3f} ms ({count / ours_mle * 1e3:.3g} fits/s), "
          f"reference kernel {ref_mle:.3f} ms ({ref_mle / ours_mle:.2f}x)")
    assert ours_findroi <= ref_findroi
    assert ours_mle <= ref_mle * 1.05
