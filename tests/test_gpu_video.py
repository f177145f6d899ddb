"""Chrono-video windows that slide by one frame (the sliding-window kernel) against the oracle
(needs a GB300).

Runs of equal-length windows (2..64 frames), each the previous one shifted by one frame, take
the kernel that keeps each pixel's window bit planes in registers and shifts one frame in per
window; the growing
and shrinking windows at the ends of a create_video sequence (src/main.rs:230-286) go to the
batched kernel. Every window must equal the oracle's composite of that window alone: the
composite and blend mask within 1 LSB per band (expected 0) and the warning count exact."""
import ctypes as ct

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

OUTLIERS = ["first", "last", "extreme", "average", "forward", "backward"]
BACKGROUNDS = ["first", "random", "average", "median"]


def run_windows(ctx, pool, wins, p, blend_offset=0):
    """cp_composite_video_device over `wins` (lists of pool indices). Returns per window
    (composite, blend mask, warnings)."""
    count, h, w, c = pool.shape
    ptrs = []
    try:
        frame_ptrs = (ct.c_void_p * count)()
        for i in range(count):
            frame_ptrs[i] = ctx.upload(pool[i])
            ptrs.append(frame_ptrs[i])
        nwin = len(wins)
        starts = np.zeros(nwin, np.int64)
        lens = np.zeros(nwin, np.int32)
        idx = []
        for k, ind in enumerate(wins):
            starts[k] = len(idx)
            lens[k] = len(ind)
            idx += list(ind)
        idx = np.asarray(idx or [0], np.int32)
        fb = h * w * c
        # one buffer for all outputs; blend_offset shifts the blend masks off 4-byte alignment
        buf = ctx.alloc(2 * nwin * fb + 64)
        ptrs.append(buf)
        outs = (ct.c_void_p * nwin)(*[buf + k * fb for k in range(nwin)])
        blends = (ct.c_void_p * nwin)(*[buf + nwin * fb + blend_offset + k * fb for k in range(nwin)])
        warn = ctx.alloc(8 * nwin)
        ptrs.append(warn)
        ctx.upload(np.zeros(nwin, np.uint64), warn)
        rc = _abi.lib().cp_composite_video_device(
            ctx.handle, frame_ptrs, count, w, h, c, nwin, starts.ctypes.data_as(_abi.I64P),
            lens.ctypes.data_as(_abi.I32P), idx.ctypes.data_as(_abi.I32P), ct.byref(p), outs,
            blends, warn, None)
        ctx.check(rc, "video")
        ctx.synchronize()
        wv = ctx.download(warn, (nwin,), np.uint64)
        return [(ctx.download(outs[k], (h, w, c)), ctx.download(blends[k], (h, w, c)), int(wv[k]))
                for k in range(nwin)]
    finally:
        for q in ptrs:
            ctx.free(q)


def check(pool, wins, p, got):
    for k, ind in enumerate(wins):
        if not ind:
            continue
        ref = oracle.composite(pool[list(ind)], p, frame_offset=ind[0], threads=8)
        cases.assert_close_u8(got[k][0], ref[0], what="window %d composite" % k)
        cases.assert_close_u8(got[k][1], ref[1], what="window %d blend" % k)
        assert got[k][2] == ref[2], "window %d warnings %d vs %d" % (k, got[k][2], ref[2])


@pytest.mark.parametrize("L", [2, 3, 8, 31, 32, 33, 64, 65, 100, 128])
def test_sliding_lengths(ctx, L):
    """Window lengths of the one- and two-word plane kernels (2..64), odd and even (median
    pairs), and longer windows (the batched kernel), on a frame whose last 32-pixel tile is
    partial."""
    rng = np.random.default_rng(L)
    nwin = 7
    pool = cases.random_stack(rng, L + nwin - 1, 13, 37, 3, n_spots=6)
    wins = [list(range(k, k + L)) for k in range(nwin)]
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                     background="first")
    check(pool, wins, p, run_windows(ctx, pool, wins, p))


@pytest.mark.parametrize("outlier", OUTLIERS)
@pytest.mark.parametrize("background", BACKGROUNDS)
def test_sliding_modes(ctx, outlier, background):
    rng = np.random.default_rng(100 + 10 * OUTLIERS.index(outlier) + BACKGROUNDS.index(background))
    L, nwin = 20, 9
    pool = cases.random_stack(rng, L + nwin - 1, 11, 64, 3, n_spots=8)
    wins = [list(range(k, k + L)) for k in range(nwin)]
    p = cases.params(mode="outlier", threshold="abs/0.04/0.25", outlier=outlier,
                     background=background, seed=11)
    check(pool, wins, p, run_windows(ctx, pool, wins, p))


def test_sliding_weights_and_unaligned_blend(ctx):
    """0/1 weights (a channel left out of the distance and the median) and blend masks off a
    4-byte boundary (byte stores)."""
    rng = np.random.default_rng(5)
    L, nwin = 12, 10
    pool = cases.random_stack(rng, L + nwin - 1, 9, 40, 3, n_spots=5)
    wins = [list(range(k, k + L)) for k in range(nwin)]
    p = cases.params(mode="outlier", threshold="abs/0.03/0.1", outlier="forward",
                     background="median", weights=[1, 0, 1, 1])
    check(pool, wins, p, run_windows(ctx, pool, wins, p, blend_offset=1))


@pytest.mark.parametrize("vin", [(0, 6, 1), (-3, 5, 1), (None, 7, 1), (0, 6, 2)])
def test_create_video_windows(ctx, vin):
    """The windows create_video makes (growing at the start, shrinking at the end, steps 1
    and 2): sliding runs and the batched kernel together."""
    rng = np.random.default_rng(9)
    count = 30
    pool = cases.random_stack(rng, count, 10, 45, 3, n_spots=7)
    wins = [ind for _, ind in cg.video_windows(count, vin)]
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="average",
                     background="first")
    check(pool, wins, p, run_windows(ctx, pool, wins, p))


def test_sliding_many_windows(ctx):
    """More windows than one launch takes (the call is split) on a small frame."""
    rng = np.random.default_rng(21)
    L, nwin = 5, 700
    pool = cases.random_stack(rng, L + nwin - 1, 4, 20, 3, n_spots=3)
    wins = [list(range(k, k + L)) for k in range(nwin)]
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                     background="first")
    check(pool, wins, p, run_windows(ctx, pool, wins, p))


def test_sliding_over_index_list(ctx):
    """Windows over an arbitrary sequence of pool frames (not consecutive indices)."""
    rng = np.random.default_rng(33)
    count, L, nwin = 40, 16, 12
    pool = cases.random_stack(rng, count, 12, 33, 3, n_spots=6)
    seq = rng.permutation(count)[: L + nwin - 1].tolist()
    wins = [seq[k:k + L] for k in range(nwin)]
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="backward",
                     background="random", seed=3)
    check(pool, wins, p, run_windows(ctx, pool, wins, p))
