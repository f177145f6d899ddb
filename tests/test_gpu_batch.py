"""The persistent batched kernel and the chrono-video entry point against the oracle
(needs a GB300). Each stack of a batch must give exactly what it gives alone."""
import ctypes as ct

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu


class DeviceStacks:
    """Frames uploaded to the device and cp_stack descriptors pointing at them."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.ptrs = []

    def upload(self, arr):
        p = self.ctx.upload(arr)
        self.ptrs.append(p)
        return p

    def alloc(self, nbytes):
        p = self.ctx.alloc(nbytes)
        self.ptrs.append(p)
        return p

    def free(self):
        for p in self.ptrs:
            self.ctx.free(p)
        self.ptrs = []


def run_batch(ctx, items):
    """items: list of (frames [n,h,w,c], params kwargs, frame_offset). Returns per-stack
    (out, blend, warnings) from one cp_composite_batch_device call."""
    ds = DeviceStacks(ctx)
    try:
        stacks = (_abi.Stack * len(items))()
        params = (_abi.Params * len(items))()
        outs = (ct.c_void_p * len(items))()
        blends = (ct.c_void_p * len(items))()
        keep = []
        shapes = []
        for i, (frames, kw, off) in enumerate(items):
            n, h, w, c = frames.shape
            base = ds.upload(frames)
            stacks[i] = _abi.Stack(n=n, width=w, height=h, channels=c, base=base,
                                   frame_stride=h * w * c, frame_offset=off)
            params[i] = cg.make_params(keep=keep, **kw)
            outs[i] = ds.alloc(h * w * c)
            blends[i] = ds.alloc(h * w * c)
            shapes.append((h, w, c))
        warn = ds.alloc(8 * len(items))
        ctx.upload(np.zeros(len(items), np.uint64), warn)
        for _ in range(2):  # the second call replays the captured graph
            rc = _abi.lib().cp_composite_batch_device(ctx.handle, stacks, params, len(items), outs,
                                                      blends, warn, None)
            ctx.check(rc, "batch")
            ctx.synchronize()
        res = []
        wv = ctx.download(warn, (len(items),), np.uint64)
        for i, shp in enumerate(shapes):
            res.append((ctx.download(outs[i], shp), ctx.download(blends[i], shp), int(wv[i]) // 2))
        return res
    finally:
        ds.free()


def test_batch_matches_oracle(ctx):
    rng = np.random.default_rng(1)
    items = []
    for n, (h, w) in [(5, (17, 29)), (16, (40, 64)), (33, (64, 64)), (64, (21, 300)), (100, (9, 77))]:
        frames = cases.random_stack(rng, n, h, w, 3, n_spots=5)
        items.append((frames, dict(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                                   background="first"), 0))
    items.append((cases.random_stack(rng, 12, 30, 30, 3), dict(mode="outlier", threshold="rel/2/4",
                                                               outlier="average", background="median"), 0))
    items.append((cases.random_stack(rng, 20, 31, 33, 3), dict(mode="darker"), 0))
    items.append((cases.random_stack(rng, 20, 31, 33, 3), dict(mode="lighter", fade="clamp/abs/0,0/9,1"), 4))
    got = run_batch(ctx, items)
    for (frames, kw, off), (out, blend, warn) in zip(items, got):
        p = cases.params(**kw)
        ref = oracle.composite(frames, p, frame_offset=off)
        cases.assert_close_u8(out, ref[0], what="batch composite")
        if kw["mode"] == "outlier":
            cases.assert_close_u8(blend, ref[1], what="batch blend")
            assert warn == ref[2]


@pytest.mark.parametrize("kw", [
    dict(threshold="abs/0.05/0.2", outlier="extreme"),
    dict(threshold="abs/0.04/0.3", outlier="average"),
    dict(threshold="abs/0.04/0.3", outlier="backward"),
    dict(threshold="rel/2/4", outlier="first"),
    dict(threshold="rel/1.5/3", outlier="average"),
    dict(threshold="rel/1.5/3", outlier="forward"),
], ids=lambda kw: kw["threshold"] + "-" + kw["outlier"])
def test_uniform_batch_variants(ctx, kw):
    """Batches whose RGB stacks share one setting (background first) run the specialised
    batched kernel of that setting; uneven frame counts and sizes still mix inside it."""
    rng = np.random.default_rng(7)
    items = []
    for n, (h, w) in [(9, (13, 40)), (32, (24, 70)), (48, (17, 129)), (64, (33, 50)), (90, (8, 60))]:
        frames = cases.random_stack(rng, n, h, w, 3, n_spots=5)
        items.append((frames, dict(mode="outlier", background="first", **kw), 0))
    got = run_batch(ctx, items)
    for (frames, k, off), (out, blend, warn) in zip(items, got):
        ref = oracle.composite(frames, cases.params(**k), frame_offset=off)
        cases.assert_close_u8(out, ref[0], what="batch composite")
        cases.assert_close_u8(blend, ref[1], what="batch blend")
        assert warn == ref[2]


def test_video_windows_match_oracle(ctx):
    """Overlapping windows over one resident pool (stride 1 and 2) with an absolute fade,
    evaluated at each window's first index."""
    rng = np.random.default_rng(2)
    count = 24
    pool = cases.random_stack(rng, count, 36, 50, 3, n_spots=8)
    ds = DeviceStacks(ctx)
    try:
        frame_ptrs = (ct.c_void_p * count)(*[ds.upload(pool[i]) for i in range(count)])
        for vin in [(0, 8, 1), (-2, 6, 2)]:
            wins = cg.video_windows(count, vin)
            nwin = len(wins)
            starts = np.zeros(nwin, np.int64)
            lens = np.zeros(nwin, np.int32)
            idx = []
            for k, (_, ind) in enumerate(wins):
                starts[k] = len(idx)
                lens[k] = len(ind)
                idx += ind
            idx = np.asarray(idx or [0], np.int32)
            keep = []
            p = cg.make_params(keep=keep, mode="outlier", threshold="abs/0.05/0.2", outlier="forward",
                               background="first", fade="repeat/abs/0,1/3,0.25")
            outs = (ct.c_void_p * nwin)(*[ds.alloc(36 * 50 * 3) for _ in range(nwin)])
            blends = (ct.c_void_p * nwin)(*[ds.alloc(36 * 50 * 3) for _ in range(nwin)])
            rc = _abi.lib().cp_composite_video_device(
                ctx.handle, frame_ptrs, count, 50, 36, 3, nwin, starts.ctypes.data_as(_abi.I64P),
                lens.ctypes.data_as(_abi.I32P), idx.ctypes.data_as(_abi.I32P), ct.byref(p), outs,
                blends, None, None)
            ctx.check(rc, "video")
            ctx.synchronize()
            for k, (_, ind) in enumerate(wins):
                if not ind:
                    continue
                ref = oracle.composite(pool[ind], p, frame_offset=ind[0])
                cases.assert_close_u8(ctx.download(outs[k], (36, 50, 3)), ref[0], what="window %d" % k)
                cases.assert_close_u8(ctx.download(blends[k], (36, 50, 3)), ref[1], what="window %d" % k)
    finally:
        ds.free()


def test_big_stacks_leave_the_batch(ctx):
    """A stack that fills the GPU alone (16 x 480x640: 2400 tiles of 128 pixels) runs on the
    pixel-thread kernel by itself, the small ones in the batched launch; every stack still
    matches the oracle and its own warnings."""
    rng = np.random.default_rng(21)
    big = cases.random_stack(rng, 16, 480, 640, 3, n_spots=6)
    small = [cases.random_stack(rng, n, h, w, 3, n_spots=3)
             for n, h, w in ((20, 40, 64), (33, 24, 48), (9, 30, 70))]
    kws = [dict(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme", background="first"),
           dict(mode="outlier", threshold="rel/2/4", outlier="average", background="first"),
           dict(mode="outlier", threshold="abs/0.05/0.2", outlier="forward", background="median"),
           dict(mode="outlier", threshold="abs/0.04", outlier="last", background="average")]
    items = [(big, kws[0], 0)] + [(f, kw, 0) for f, kw in zip(small, kws[1:])]
    counts0 = ct.c_uint64()
    ctx.check(_abi.lib().cp_ctx_launch_counts(ctx.handle, ct.byref(counts0), None, None))
    got = run_batch(ctx, items)
    counts1 = ct.c_uint64()
    ctx.check(_abi.lib().cp_ctx_launch_counts(ctx.handle, ct.byref(counts1), None, None))
    assert counts1.value - counts0.value >= 2  # the big stack alone, then the batch
    for (frames, kw, off), (o, b, wn) in zip(items, got):
        p = cases.params(**kw)
        ref = oracle.composite(frames, p, threads=8)
        cases.assert_close_u8(o, ref[0], what="%s composite" % kw)
        cases.assert_close_u8(b, ref[1], what="%s blend" % kw)
        assert wn == ref[2]
