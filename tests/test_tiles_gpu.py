"""Sub-region tiling on the GPU against the reference restatement
(oracle/tiles_port.py): bit-identical sub-regions, overlap removal and
stitched images."""
import numpy as np
import pytest

from bamf_gb300 import tiles
from oracle import tiles_port

pytestmark = pytest.mark.gpu

GEOMS = [(256, 256, 3, 10, 3), (37, 50, 2, 8, 2), (16, 16, 2, 16, 3), (20, 9, 3, 4, 1), (64, 48, 1, 16, 0)]


@pytest.mark.parametrize("Y,X,Z,B,O", GEOMS)
def test_make_subregions_matches_reference(cuda_lib, Y, X, Z, B, O):
    rng = np.random.default_rng(Y * 7 + X)
    D = rng.poisson(30, size=(Y, X, Z)).astype(np.float32)
    V = rng.random((Y, X)).astype(np.float32)
    R, S, RV = tiles.makeSubRegions(D, B, O, V)
    R0, S0, RV0 = tiles_port.make_sub_regions(D, B, O, V)
    np.testing.assert_array_equal(R, R0)
    np.testing.assert_array_equal(RV, RV0)
    for k in ("Xsize", "Ysize", "FrameNum", "ROI_Ind"):
        np.testing.assert_array_equal(S[k], S0[k])
    assert (S["Xsub"], S["Ysub"]) == (S0["Xsub"], S0["Ysub"])


def test_packed_layout_is_each_subregion_with_its_own_height(cuda_lib):
    import torch
    Y, X, Z, B, O = 37, 50, 2, 8, 2
    D = np.random.default_rng(1).random((Y, X, Z)).astype(np.float32)
    R0, S0, _ = tiles_port.make_sub_regions(D, B, O)
    r = tiles.make_subregions_device(torch.from_numpy(D.ravel(order="F")).cuda(), Y, X, Z, B, O, packed=True)
    data = r["data"].cpu().numpy()
    T = B + 2 * O
    for k in range(r["n"]):
        ny, nx = int(S0["Ysize"][k]), int(S0["Xsize"][k])
        got = data[k * T * T:k * T * T + ny * nx].reshape(nx, ny).T
        np.testing.assert_array_equal(got, R0[:ny, :nx, k])


@pytest.mark.parametrize("Y,X,Z,B,O", GEOMS)
@pytest.mark.parametrize("zoom", [1, 3])
def test_remove_overlapping_and_stitch_match_reference(cuda_lib, Y, X, Z, B, O, zoom):
    rng = np.random.default_rng(Y + X + zoom)
    D = np.zeros((Y, X, Z), np.float32)
    _, S, _ = tiles_port.make_sub_regions(D, B, O)
    T = B + 2 * O
    n = S["Xsub"] * S["Ysub"] * Z
    G = rng.random((zoom * T, zoom * T, n)).astype(np.float32)
    M = tiles.removeOverlapping(S, O, zoom, G)
    M0 = tiles_port.remove_overlapping(S, O, zoom, G)
    np.testing.assert_array_equal(M, M0)
    for src in (M0, G):  # after overlap removal, and raw (overlaps summed in ROI order)
        F = tiles.stitchROIs(src, S, O, [Y, X, Z], B, zoom)
        F0 = tiles_port.stitch_rois(src, S, O, [Y, X, Z], B, zoom)
        np.testing.assert_array_equal(F, F0)


def test_stitch_flags_duplicate_subregions(cuda_lib):
    Y, X, B, O = 30, 30, 10, 3
    _, S, _ = tiles_port.make_sub_regions(np.zeros((Y, X, 1), np.float32), B, O)
    S2 = dict(S)
    for k in ("Xsize", "Ysize", "FrameNum", "ROI_Ind"):
        S2[k] = np.concatenate([S[k], S[k][:1]])
    G = np.ones((B + 2 * O, B + 2 * O, len(S2["Xsize"])), np.float32)
    with pytest.raises(ValueError):
        tiles.stitchROIs(G, S2, O, [Y, X, 1], B, 1)
