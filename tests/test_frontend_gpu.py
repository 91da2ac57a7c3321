"""GPU parity of the front end.

findROI: the maxima coordinates (order included), box corners and ROI
crops are bit-exact against the CPU restatement of the reference kernels and
findROI.m glue.  gaussMLE: parameters within 1e-4 relative of the float
restatement of kernel_MLEFit_XYNB_; the error against the FP64 restatement
is measured and bounded."""
import numpy as np
import pytest

import oracle
from bamf_gb300 import frontend, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def frames():
    st, truth = synth.frames(12, seed=1)
    return st, truth


def test_findroi_coords_bit_exact(cuda_lib, frames):
    st, _ = frames
    ref = oracle.findroi(st, 1.3, 2.6, 7)
    SMD, rois, coords = frontend.findROI(st, 1.3, 2.6, 7)
    np.testing.assert_array_equal(coords, ref["coords"])
    np.testing.assert_array_equal(SMD["XBoxCorner"], ref["XBoxCorner"])
    np.testing.assert_array_equal(SMD["YBoxCorner"], ref["YBoxCorner"])
    np.testing.assert_array_equal(rois, ref["ROIStack"])


def test_findroi_boxsize8_findpriors_settings(cuda_lib, frames):
    """findPriors.m:35-39: Boxsize 8, Minval = MeanPhotons/(4 pi s^2)/4."""
    st, _ = frames
    minval = 1500 / (4 * np.pi * 1.3 ** 2) / 4
    ref = oracle.findroi(st[:, :, :5], 1.3, 2.6, 8, minval)
    _, rois, coords = frontend.findROI(st[:, :, :5], 1.3, 2.6, 8, minval)
    np.testing.assert_array_equal(coords, ref["coords"])
    np.testing.assert_array_equal(rois, ref["ROIStack"])


def test_findroi_deep_stack_float_window_bounds(cuda_lib):
    """300 frames of 256x256: from frame 256 on, the row-max window bounds
    are rounded in float exactly as the reference kernel forms them."""
    st, _ = synth.frames(300, seed=5)
    ref = oracle.findroi(st, 1.3, 2.6, 7, threads=16)
    _, _, coords = frontend.findROI(st, 1.3, 2.6, 7)
    np.testing.assert_array_equal(coords, ref["coords"])


def test_findroi_small_and_edge_frames(cuda_lib):
    rng = np.random.default_rng(3)
    st = rng.poisson(20, size=(32, 32, 3)).astype(np.float32)
    st[3, 4, 0] += 900
    st[30, 31, 1] += 900   # near the edge: clamped box
    st[0, 0, 2] += 900     # corner
    ref = oracle.findroi(st, 1.3, 2.6, 7)
    SMD, rois, coords = frontend.findROI(st, 1.3, 2.6, 7)
    np.testing.assert_array_equal(coords, ref["coords"])
    np.testing.assert_array_equal(SMD["XBoxCorner"], ref["XBoxCorner"])
    np.testing.assert_array_equal(SMD["YBoxCorner"], ref["YBoxCorner"])
    np.testing.assert_array_equal(rois, ref["ROIStack"])
    assert len(coords) >= 3


@pytest.mark.parametrize("boxsize", [3, 12, 13])
def test_findroi_boxsizes_on_both_maxima_kernels(cuda_lib, boxsize):
    """Boxsize 3 and 12 take the wide maxima kernel with k chosen at run time
    (7 and 8 have their own instantiations), 13 the 32-column kernel: the
    same coordinates and crops as the oracle."""
    st, _ = synth.frames(6, seed=11)
    ref = oracle.findroi(st, 1.3, 2.6, boxsize)
    SMD, rois, coords = frontend.findROI(st, 1.3, 2.6, boxsize)
    assert len(coords) > 3
    np.testing.assert_array_equal(coords, ref["coords"])
    np.testing.assert_array_equal(SMD["XBoxCorner"], ref["XBoxCorner"])
    np.testing.assert_array_equal(rois, ref["ROIStack"])


@pytest.mark.parametrize("shape", [(320, 320), (250, 96), (96, 250), (33, 47)])
def test_findroi_frame_shapes_on_both_filter_paths(cuda_lib, shape):
    """Frames whose intermediate images do not fit the fused filter's slot
    (320 x 320) take the row / column kernels; the others, with rows and
    columns not multiples of the tile sizes and unaligned row lengths, take
    the fused filter.  Both are bit-exact against the oracle."""
    ys, xs = shape
    st, _ = synth.frames(3, size=max(ys, xs), seed=6)
    st = np.asfortranarray(st[:ys, :xs, :])
    ref = oracle.findroi(st, 1.3, 2.6, 7)
    SMD, rois, coords = frontend.findROI(st, 1.3, 2.6, 7)
    assert len(coords) > 3
    np.testing.assert_array_equal(coords, ref["coords"])
    np.testing.assert_array_equal(SMD["XBoxCorner"], ref["XBoxCorner"])
    np.testing.assert_array_equal(rois, ref["ROIStack"])


def test_gaussmle_matches_float_restatement_and_fp64(cuda_lib, frames):
    st, _ = frames
    _, rois, _ = frontend.findROI(st, 1.3, 2.6, 7)
    for it in (10, 20):
        res = frontend.gaussMLE(rois, "Basic", "CCD", 1.3, Iterations=it)
        P = np.stack([res["Y"], res["X"], res["Photons"], res["BG"]], 1)
        ref = oracle.gaussmle(rois, 1.3, it)
        ref64 = oracle.gaussmle(rois, 1.3, it, double=True)
        rel = np.abs(P - ref["P"]) / np.maximum(np.abs(ref["P"]), 1e-3)
        assert np.percentile(rel, 99.9) < 1e-4, np.percentile(rel, 99.9)
        rel64 = np.abs(P - ref64["P"]) / np.maximum(np.abs(ref64["P"]), 1e-3)
        assert np.median(rel64) < 1e-5 and np.percentile(rel64, 99) < 1e-3
        crlb = np.stack([res["Y_SE"], res["X_SE"], res["Photons_SE"], res["BG_SE"]], 1) ** 2
        good = np.isfinite(ref["CRLB"]).all(1) & (ref["CRLB"] > 0).all(1)
        relc = np.abs(crlb[good] - ref["CRLB"][good]) / np.abs(ref["CRLB"][good])
        assert np.percentile(relc, 99) < 1e-3
        np.testing.assert_allclose(res["LogLikelihood"], ref["LL"], rtol=1e-3, atol=1e-2)


@pytest.mark.parametrize("chunk", [64, 37])
def test_findroi_from_pinned_host_in_chunks_matches_the_device_call(cuda_lib, chunk):
    """bamf_find_roi_pinned (frames copied in chunks, each chunk's filters
    started as it lands) gives the device call's outputs bit for bit, on a
    300-frame stack whose row-max window bounds round from frame 256 on."""
    import torch
    st, _ = synth.frames(300, seed=5)
    host = torch.from_numpy(np.asfortranarray(st).ravel(order="F")).pin_memory()
    fr = frontend.FindRoiDevice()
    a = fr.run(host.cuda(), 256, 256, 300, boxsize=7)
    b = fr.run_pinned(host, 256, 256, 300, boxsize=7, chunk_frames=chunk)
    torch.cuda.synchronize()
    c = int(a["count"].item())
    assert c > 0 and int(b["count"].item()) == c
    assert torch.equal(a["coords"][:c], b["coords"][:c])
    assert torch.equal(a["corners"][:c], b["corners"][:c])
    assert torch.equal(a["stack"][:c], b["stack"][:c])
    assert torch.equal(b["frames"], host.cuda())


@pytest.mark.parametrize("chunk,cap_less", [(64, 0), (37, 25)])
def test_findroi_fit_pinned_equals_the_separate_calls(cuda_lib, chunk, cap_less):
    """bamf_find_roi_fit_pinned (each chunk's maxima compacted, cropped and
    fitted once its frames are done) gives the coordinates, corners, crops
    and count of bamf_find_roi_pinned and the fits of gaussMLE on that ROI
    stack, bit for bit, on a 300-frame stack whose row-max window bounds
    round; with a capacity below the count only the first `capacity` ROIs
    are written and fitted."""
    import torch
    st, _ = synth.frames(300, seed=5)
    host = torch.from_numpy(np.asfortranarray(st).ravel(order="F")).pin_memory()
    fr = frontend.FindRoiDevice()
    a = fr.run_pinned(host, 256, 256, 300, boxsize=7, chunk_frames=chunk)
    torch.cuda.synchronize()
    c = int(a["count"].item())
    assert c > 100
    cap = c - cap_less
    b = fr.run_fit_pinned(host, 256, 256, 300, boxsize=7, psf_sigma=1.3, iterations=10, chunk_frames=chunk,
                          capacity=cap)
    torch.cuda.synchronize()
    assert int(b["count"].item()) == c
    assert torch.equal(a["coords"][:cap], b["coords"][:cap])
    assert torch.equal(a["corners"][:cap], b["corners"][:cap])
    assert torch.equal(a["stack"][:cap], b["stack"][:cap])
    P, CR, LL = frontend.gauss_mle_device(a["stack"][:cap].contiguous(), 7, cap, 1.3, 10)
    torch.cuda.synchronize()
    assert torch.equal(P.view(4, cap), b["P"][:, :cap])
    assert torch.equal(CR.view(4, cap), b["CR"][:, :cap])
    assert torch.equal(LL, b["LL"][:cap])
