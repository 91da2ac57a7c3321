"""The difference-of-Gaussians stage of findROI on the GPU against the
oracle, bit for bit (bamf_find_roi_dog_device): ordinary frames, frames
whose recurrences reach tiny or huge values (where the filters fall back from
the fast division by b0 to IEEE division), negative and signed-zero pixels,
odd shapes on the fused filter and a frame too large for its slot.  And the
fast division itself against IEEE division over every float."""
import numpy as np
import pytest

import oracle
from bamf_gb300 import frontend, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sigma", [0.8, 1.3, 2.0, 2.6, 3.9, 5.2])
def test_fast_division_equals_ieee_division_on_every_float(cuda_lib, sigma):
    r = frontend.division_check(sigma, device=True)
    print(sigma, r)
    assert r["host_exact"]
    assert r["dev_mismatch_in_range"] == 0
    # outside [2^-100, 2^100] the fast sequence does differ (subnormal
    # residuals, infinities): those q take IEEE division
    assert r["dev_mismatch"] > 0


def _frames(case):
    rng = np.random.default_rng(8)
    if case == "synth":
        st, _ = synth.frames(4, seed=2)
        return st
    if case == "zero_background":
        st = np.zeros((256, 256, 3), np.float32, order="F")
        for z in range(3):
            for _ in range(12):
                y, x = rng.integers(4, 252, 2)
                st[y - 1:y + 2, x - 1:x + 2, z] = rng.uniform(200, 2000)
        return st
    if case == "tiny":
        st, _ = synth.frames(2, size=96, seed=3)
        return np.asfortranarray(st * np.float32(1e-30))
    if case == "huge":
        st, _ = synth.frames(2, size=96, seed=4)
        return np.asfortranarray(st * np.float32(1e31))
    if case == "signed":
        st, _ = synth.frames(2, size=96, seed=5)
        st = np.asfortranarray(st - np.float32(40.0))
        st[st == 0] = -0.0
        st[:10, :, 0] = -0.0
        return st
    if case == "odd_shape":
        st, _ = synth.frames(3, size=64, seed=6)
        return np.asfortranarray(st[:47, :33, :])
    if case == "large_frame":
        st, _ = synth.frames(2, size=320, seed=7)
        return st
    raise ValueError(case)


@pytest.mark.parametrize("case", ["synth", "zero_background", "tiny", "huge", "signed", "odd_shape", "large_frame"])
def test_dog_bit_exact_against_the_oracle(cuda_lib, case):
    import torch
    st = _frames(case)
    ys, xs, zs = st.shape
    want = oracle.findroi_dog(st, 1.3, 2.6)
    flat = torch.from_numpy(np.ascontiguousarray(np.asarray(st, np.float32).ravel(order="F"))).cuda()
    fr = frontend.FindRoiDevice()
    got = fr.dog(flat, ys, xs, zs, 1.3, 2.6)
    torch.cuda.synchronize()
    got = got.cpu().numpy()
    bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
    assert bad.size == 0, (bad.size, bad[:5], got[bad[:5]], want[bad[:5]])
