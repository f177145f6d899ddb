"""Camera-shake search on the GPU against the oracle (needs a GB300): per-frame offsets and
every wrapping-i32 sum bit-exact (src/shake.rs:190-385)."""
import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi, example_data
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_shake_offsets_and_sums(ctx):
    frames, shifts = example_data.shake_stack(seed=5, n=6, w=320, h=240, max_shift=4, n_disks=1,
                                               rmin=6, rmax=8)
    anchors = [(80, 70), (240, 70), (80, 170), (240, 170)]
    got_offs, got_d = ctx.shake_analyze(frames, anchors, 10, 8, diffs=True)
    ref_offs, ref_d = oracle.shake(frames, anchors, 10, 8, threads=8, diffs=True)
    assert np.array_equal(got_d, ref_d)
    assert np.array_equal(got_offs, ref_offs)
    # frame i shows the background window at shifts[i], so frame 0's anchor content sits at
    # an offset of t_0 - t_i in frame i
    assert np.array_equal(got_offs, shifts[0] - shifts)


@pytest.mark.parametrize("c", [1, 3, 4])
def test_shake_channels_and_ties(ctx, c):
    rng = np.random.default_rng(c)
    frames = rng.integers(0, 256, size=(4, 60, 70, c), dtype=np.uint8)
    frames[2] = frames[0]  # exact match at offset 0 for frame 2
    flat = np.full((3, 40, 40, c), 9, np.uint8)  # all sums equal: first minimum
    for f, anchors, r, s in [(frames, [(30, 30), (40, 25)], 4, 5), (flat, [(20, 20)], 3, 4)]:
        got_o, got_d = ctx.shake_analyze(f, anchors, r, s, diffs=True)
        ref_o, ref_d = oracle.shake(f, anchors, r, s, diffs=True)
        assert np.array_equal(got_d, ref_d) and np.array_equal(got_o, ref_o)


def test_shake_wrapping(ctx):
    r, s = 53, 1
    size = 2 * r + 1
    h = w = size + 2 * s + 2
    f0 = np.zeros((h, w, 3), np.uint8)
    f1 = np.full((h, w, 3), 255, np.uint8)
    f1[0, 0] = 0
    frames = np.stack([f0, f1])
    got_o, got_d = ctx.shake_analyze(frames, [(w // 2, h // 2)], r, s, diffs=True)
    ref_o, ref_d = oracle.shake(frames, [(w // 2, h // 2)], r, s, diffs=True)
    assert np.array_equal(got_d, ref_d) and np.array_equal(got_o, ref_o)


def test_shake_out_of_range(ctx):
    frames = np.zeros((2, 50, 50, 3), np.uint8)
    with pytest.raises(_abi.ChronoError) as e:
        ctx.shake_analyze(frames, [(5, 25)], 4, 6)
    assert e.value.status == _abi.CP_ERR_RANGE


def test_shaken_stack_composite(ctx):
    """Shake offsets -> Crop::create -> composite with per-frame address offsets, against
    the oracle on the same crops."""
    frames, _ = example_data.shake_stack(seed=8, n=10, w=256, h=160, max_shift=3, n_disks=2,
                                          rmin=8, rmax=12)
    anchors = [(64, 50), (190, 50), (64, 110), (190, 110)]
    offs = ctx.shake_analyze(frames, anchors, 8, 7)
    crops = cg.Crop.create(offs, 256, 160)
    assert crops is not None
    size = (int(crops[0, 2]), int(crops[0, 3]))
    keep = []
    p = cg.make_params(keep=keep, mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                       background="first")
    got = ctx.composite(frames, p, crop=(crops[:, :2], size))
    ref = oracle.composite(frames, p, crop=crops[:, :2], out_size=size)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
