"""The reference's sub-region tiling restated (oracle/tiles_port.py): the
properties the reference's geometry has, on small cases."""
import numpy as np
import pytest

from oracle import tiles_port


def test_subregions_cover_the_frame_and_interiors_partition_it():
    rng = np.random.default_rng(0)
    for (Y, X, B, O) in [(256, 256, 10, 3), (37, 50, 8, 2), (16, 16, 16, 3), (20, 9, 4, 1)]:
        D = rng.random((Y, X, 2)).astype(np.float32)
        R, S, _ = tiles_port.make_sub_regions(D, B, O)
        assert R.shape[2] == S["Xsub"] * S["Ysub"] * 2
        # zoom 1 grids = the data: removeOverlapping + stitch gives the frames back
        M = tiles_port.remove_overlapping(S, O, 1, R)
        F = tiles_port.stitch_rois(M, S, O, [Y, X, 2], B, 1)
        np.testing.assert_array_equal(F, D)


def test_stitch_without_overlap_removal_counts_the_overlaps():
    Y, X, B, O = 30, 30, 10, 3
    D = np.ones((Y, X, 1), np.float32)
    R, S, _ = tiles_port.make_sub_regions(D, B, O)
    F = tiles_port.stitch_rois(R, S, O, [Y, X, 1], B, 1)[:, :, 0]
    assert F[0, 0] == 1 and F[15, 15] == 1
    assert F[10, 5] == 2 and F[10, 10] == 4   # inside two / four sub-regions


def test_circle_example_fixture_shapes():
    """tests/golden/circle_example.npz (the reference's CircleData example,
    first 400 frames): 10 x 10 frames, ground truth of those frames only."""
    import os
    f = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "circle_example.npz"))
    assert f["data"].shape == (10, 10, 400) and f["data"].dtype == np.float32
    fn = f["frame_num"]
    assert fn.min() >= 1 and fn.max() <= 400
    assert len(f["x"]) == len(f["y"]) == len(fn) == 1799
    assert float(f["psf_sigma"]) == pytest.approx(1.2) and float(f["bg"]) == 20.0
    assert (f["x"] > 0).all() and (f["x"] < 11).all() and (f["y"] > 0).all() and (f["y"] < 11).all()
