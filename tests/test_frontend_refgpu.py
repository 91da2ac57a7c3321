"""The front end against the reference's own CUDA kernels (compiled
unmodified for sm_103a into oracle/_ref by `make -C oracle ref-cubin`, run
with the reference's launch geometry by oracle/refgpu.py): the maxima flags
must be identical, and the gaussMLE parameters within 1e-4 relative.
Skipped where the cubins were not built (no reference tree)."""
import numpy as np
import pytest

from oracle import refgpu

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(not refgpu.available("findroi"), reason="reference FindROI cubin not built")
@pytest.mark.parametrize("nframes,box,minval", [(12, 7, None), (6, 8, 1500 / (4 * np.pi * 1.3 ** 2) / 4),
                                                (300, 7, None), (1100, 7, None), (300, 12, None),
                                                (300, 3, None), (40, 13, None)])
def test_findroi_flags_identical_to_reference_kernels(cuda_lib, nframes, box, minval):
    import torch
    from bamf_gb300 import frontend, synth
    st, _ = synth.frames(nframes, seed=9)
    flat = torch.from_numpy(np.ascontiguousarray(st.ravel(order="F"))).cuda()
    mv = frontend.default_minval() if minval is None else minval
    ref = refgpu.findroi_flags(flat, 256, 256, nframes, 1.3, 2.6, box, float(np.float32(mv)))
    f = frontend.FindRoiDevice()
    out = f.run(flat, 256, 256, nframes, 1.3, 2.6, box, mv, want_flags=True, want_stack=False)
    torch.cuda.synchronize()
    got = out["flags"].cpu().numpy()
    want = ref.cpu().numpy()
    assert set(np.unique(want)) <= {0.0, 1.0}
    bad = np.flatnonzero(got != (want != 0))
    assert bad.size == 0, f"{bad.size} flags differ, first at {bad[:5]}"
    assert int(out["count"].item()) == int(want.sum())


@pytest.mark.skipif(not refgpu.available("gaussmle"), reason="reference gaussMLE cubin not built")
@pytest.mark.parametrize("iterations", [10, 20])
def test_gaussmle_within_1e4_of_reference_kernel(cuda_lib, iterations):
    import torch
    from bamf_gb300 import frontend, synth
    st, _ = synth.frames(20, seed=4)
    SMD, rois, coords = frontend.findROI(st, 1.3, 2.6, 7)
    n = rois.shape[2]
    flat = torch.from_numpy(np.ascontiguousarray(rois.ravel(order="F"))).cuda()
    P, CR, LL = frontend.gauss_mle_device(flat, 7, n, 1.3, iterations)
    Pr, CRr, LLr = refgpu.gaussmle_xynb(flat, 7, n, 1.3, iterations)
    P, Pr = P.cpu().numpy().reshape(4, n), Pr.cpu().numpy().reshape(4, n)
    rel = np.abs(P - Pr) / np.maximum(np.abs(Pr), 1e-3)
    assert rel.max() < 1e-4, (rel.max(), np.unravel_index(rel.argmax(), rel.shape))
    CR, CRr = CR.cpu().numpy().reshape(4, n), CRr.cpu().numpy().reshape(4, n)
    good = np.isfinite(CRr) & (CRr > 0)
    assert (np.abs(CR[good] - CRr[good]) / CRr[good]).max() < 1e-3
    np.testing.assert_allclose(LL.cpu().numpy(), LLr.cpu().numpy(), rtol=1e-3, atol=1e-2)
