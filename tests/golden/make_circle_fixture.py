"""Writes tests/golden/circle_example.npz from the reference's own example
dataset (Examples/Circle/CircleData.mat, loaded by
Examples/Example_SyntheticCircle.m; MIT licence, (c) 2022 MohamadFazel):
the first NF frames of `Data` (10 x 10 pixels, gain 1, offset 0, PSF sigma
1.2 px, background 20 photons/pixel) and the ground-truth emitters of those
frames from `SMD` (FrameNum, X, Y, Photons).

Run in a checkout next to the reference:
    python tests/golden/make_circle_fixture.py /path/to/reference
"""
import os
import sys

import numpy as np
import scipy.io as sio

NF = 400


def main(ref: str) -> None:
    d = sio.loadmat(os.path.join(ref, "Examples", "Circle", "CircleData.mat"))
    data = np.asarray(d["Data"], np.float32)[:, :, :NF]
    smd = d["SMD"][0, 0]
    fn = np.asarray(smd["FrameNum"]).ravel().astype(np.int32)
    keep = fn <= NF
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "circle_example.npz")
    np.savez_compressed(out, data=data, frame_num=fn[keep],
                        x=np.asarray(smd["X"], np.float64).ravel()[keep],
                        y=np.asarray(smd["Y"], np.float64).ravel()[keep],
                        photons=np.asarray(smd["Photons"], np.float64).ravel()[keep],
                        psf_sigma=np.float64(np.asarray(smd["PSFSigma"]).ravel()[0]),
                        bg=np.float64(np.asarray(smd["Bg"]).ravel()[0]))
    print(out, data.shape, int(keep.sum()), "emitters")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BAMF_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_circle_fixture.py <reference tree>  (or set BAMF_REFERENCE_DIR)")
    main(ref)
