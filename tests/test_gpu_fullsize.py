"""The benchmark configurations at full size on the GPU (needs a GB300), checked through
properties that hold at any size.

A composite pixel depends only on that pixel's samples (and, for an absolute fade, the frame
indices), so the oracle run on a band of rows of the same frames gives exactly those rows of
the full-size composite. Each test launches a whole configuration — the 64 x 1920x1080 HD
stack, the 300-frame chrono-video pool with its 269 windows, the 100 x 6000x4000 shake stack —
and compares bands spread over the image (and where the outliers are) with the oracle:
composite and blend mask within 1 LSB, medians, quartiles, outlier flags and indices exact.
Whole-image properties: the host-memory and device-resident entry points agree exactly, the
warning count equals the number of all-outlier pixels, and the shake search recovers the
generated translations exactly."""
import ctypes as ct

import numpy as np
import pytest

from chrono_photo_gb300 import _abi, example_data
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

W, H, C = 1920, 1080, 3
FIXED_ROWS = [0, 1, 2, 3, 269, 270, 538, 539, 540, 541, 808, 1076, 1077, 1078, 1079]
HD_SETTINGS = [
    dict(mode="outlier", threshold="abs/0.05/0.2", outlier="average", background="first"),
    dict(mode="outlier", threshold="abs/0.05/0.2", outlier="forward", background="first"),
    dict(mode="outlier", threshold="abs/0.05/0.2", outlier="backward", background="first"),
    dict(mode="outlier", threshold="rel/3/6", outlier="average", background="first"),
    dict(mode="darker"),
    dict(mode="lighter"),
    # beyond the benchmark's six: the other pick and background modes at full size
    dict(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme", background="average"),
    dict(mode="outlier", threshold="rel/2/5", outlier="last", background="median"),
]
DEBUG_KEYS = ("median", "outlier_bits", "chosen", "background", "n_outliers")


def _ids(kw):
    return "-".join(str(v).replace("/", "_") for v in kw.values())


@pytest.fixture(scope="module")
def hd():
    """The benchmark's HD stack: 64 frames of 1920x1080 RGB (seed 2)."""
    return example_data.hd_stack(seed=2)


def _busiest_rows(n_outliers, k=4):
    """The k rows with the most outlier flags (the moving disks' paths)."""
    return np.argsort(n_outliers.sum(axis=1))[-k:].tolist()


def _check_band(got, ref, rows, outlier, rel):
    cases.assert_close_u8(got[0][rows], ref[0], what="composite")
    if not outlier:
        return
    cases.assert_close_u8(got[1][rows], ref[1], what="blend mask")
    g, r = got[3], ref[3]
    for k in DEBUG_KEYS:
        assert np.array_equal(g[k][rows], r[k]), k
    if rel:
        assert np.array_equal(g["q1"][rows], r["q1"]) and np.array_equal(g["q3"][rows], r["q3"])


@pytest.mark.parametrize("kw", HD_SETTINGS, ids=_ids)
def test_hd_stack_rows_match_oracle(ctx, hd, kw):
    p = cases.params(**kw)
    outlier = kw["mode"] == "outlier"
    got = ctx.composite(hd, p, debug=outlier)
    rows = sorted(set(FIXED_ROWS) | set(_busiest_rows(got[3]["n_outliers"]) if outlier else []))
    band = np.ascontiguousarray(hd[:, rows])
    ref = oracle.composite(band, p, debug=outlier, threads=8)
    _check_band(got, ref, rows, outlier, outlier and "rel" in kw["threshold"])
    if outlier:
        assert got[3]["n_outliers"].max() > 0, "the stack has outliers"
        if kw["background"] == "first":  # a warning per pixel whose every frame is an outlier
            assert got[2] == int((got[3]["n_outliers"] == hd.shape[0]).sum())


def test_hd_device_entry_point_equals_host(ctx, hd):
    """cp_composite_device on resident frames == cp_composite from host memory, every pixel."""
    p = cases.params(**HD_SETTINGS[0])
    host_out, host_blend, _ = ctx.composite(hd, p)
    dev = ctx.upload(hd)
    out = ctx.alloc(W * H * C)
    blend = ctx.alloc(W * H * C)
    try:
        st = _abi.Stack(n=hd.shape[0], width=W, height=H, channels=C, base=dev,
                        frame_stride=W * H * C)
        ctx.check(_abi.lib().cp_composite_device(ctx.handle, ct.byref(st), ct.byref(p), out,
                                                 blend, None, None, None), "device")
        ctx.synchronize()
        assert np.array_equal(ctx.download(out, (H, W, C)), host_out)
        assert np.array_equal(ctx.download(blend, (H, W, C)), host_blend)
    finally:
        for q in (dev, out, blend):
            ctx.free(q)


def test_hd_multi_settings_equal_single_calls(ctx, hd):
    """The benchmark's six settings in one cp_composite_multi call (the stack uploaded once)
    equal six cp_composite calls, every pixel, warnings included."""
    ps = [cases.params(**kw) for kw in HD_SETTINGS[:6]]
    for p, (o, b, wn) in zip(ps, ctx.composite_multi(hd, ps)):
        ref = ctx.composite(hd, p)
        assert np.array_equal(o, ref[0])
        assert (b is None and ref[1] is None) or np.array_equal(b, ref[1])
        assert wn == ref[2]


VIDEO_ROWS = [0, 1, 134, 270, 405, 539, 540, 675, 810, 945, 1078, 1079]


def test_video_pool_all_windows_match_oracle(ctx):
    """chrono-video at full size: 300 resident 1080p frames, the 269 windows [k, k + 32) in one
    cp_composite_video_device call (abs/0.05/0.2 extreme, background first, an absolute fade
    so that each window's frame indices matter); every window's rows against the oracle."""
    n_pool, win = 300, 32
    nwin = n_pool - win + 1
    fb = W * H * C
    pool = example_data.video_stack(seed=3, n=n_pool)
    base = ctx.upload(pool)
    outs_dev = ctx.alloc(2 * nwin * fb)
    try:
        frame_ptrs = (ct.c_void_p * n_pool)(*[base + i * fb for i in range(n_pool)])
        starts = np.arange(nwin, dtype=np.int64) * win
        lens = np.full(nwin, win, np.int32)
        idx = np.concatenate([np.arange(k, k + win, dtype=np.int32) for k in range(nwin)])
        outs = (ct.c_void_p * nwin)(*[outs_dev + k * fb for k in range(nwin)])
        blends = (ct.c_void_p * nwin)(*[outs_dev + (nwin + k) * fb for k in range(nwin)])
        p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                         background="first", fade="repeat/abs/0,1/40,0.5/80,1")
        ctx.check(_abi.lib().cp_composite_video_device(
            ctx.handle, frame_ptrs, n_pool, W, H, C, nwin, starts.ctypes.data_as(_abi.I64P),
            lens.ctypes.data_as(_abi.I32P), idx.ctypes.data_as(_abi.I32P), ct.byref(p), outs,
            blends, None, None), "cp_composite_video_device")
        ctx.synchronize()
        band = np.ascontiguousarray(pool[:, VIDEO_ROWS])
        worst = 0
        for k in range(nwin):
            ref = oracle.composite(band[k:k + win], p, frame_offset=k, threads=8)
            got_o = np.stack([ctx.download(outs[k] + r * W * C, (W, C)) for r in VIDEO_ROWS])
            got_b = np.stack([ctx.download(blends[k] + r * W * C, (W, C)) for r in VIDEO_ROWS])
            worst = max(worst, cases.assert_close_u8(got_o, ref[0], what="window %d" % k)[0],
                        cases.assert_close_u8(got_b, ref[1], what="window %d mask" % k)[0])
        assert worst <= 1
    finally:
        ctx.free(outs_dev)
        ctx.free(base)


def test_shake_full_size(ctx):
    """Camera shake at full size: 100 frames of 6000x4000 generated on the device. The search
    (4 anchors, radius 32, search radius 20) recovers the generated translations exactly; its
    SSD surfaces of three frames equal the oracle's bit for bit (wrapping i32); the composite
    of the cropped stack matches the oracle on bands of output rows, each band rebuilt from
    the source rows and columns that the per-frame crop origins select."""
    import torch
    n, w, h, r, s = 100, 6000, 4000, 32, 20
    frames, shifts = example_data.shake_stack_device(n, w, h, 12, seed=5)
    fb = w * h * C
    ptrs = (ct.c_void_p * n)(*[frames.data_ptr() + i * fb for i in range(n)])
    anchors = np.array([[1000, 800], [5000, 800], [1000, 3200], [5000, 3200]], np.int32)
    offs = np.zeros((n, 2), np.int32)
    S = 2 * s + 1
    diffs = np.zeros((n - 1, S, S), np.int32)
    ctx.check(_abi.lib().cp_shake_analyze_device(
        ctx.handle, ptrs, n, w, h, C, anchors.ctypes.data_as(_abi.I32P), len(anchors), r, s,
        offs.ctypes.data_as(_abi.I32P), diffs.ctypes.data_as(_abi.I32P)), "shake")
    assert np.array_equal(offs, shifts[0] - shifts)
    for k in (1, 50, n - 1):
        pair = frames[[0, k]].cpu().numpy()
        ref_offs, ref_diffs = oracle.shake(pair, anchors, r, s, threads=8, diffs=True)
        assert np.array_equal(ref_diffs[0], diffs[k - 1]), "SSD surface of frame %d" % k
        assert np.array_equal(ref_offs[1], offs[k])

    has_crop = ct.c_int32()
    crops = np.zeros((n, 4), np.int32)  # per frame (x, y, width, height)
    ctx.check(_abi.lib().cp_crop_create(offs.ctypes.data_as(_abi.I32P), n, w, h,
                                        ct.byref(has_crop), crops.ctypes.data_as(_abi.I32P)),
              "crop")
    assert has_crop.value
    cw, ch = int(crops[0, 2]), int(crops[0, 3])
    origins = np.ascontiguousarray(crops[:, :2])
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                     background="first")
    st = _abi.Stack(n=n, width=cw, height=ch, channels=C,
                    frames=ct.cast(ptrs, ct.POINTER(ct.c_void_p)),
                    crop=origins.ctypes.data_as(_abi.I32P), src_width=w, src_height=h)
    out = ctx.alloc(cw * ch * C)
    blend = ctx.alloc(cw * ch * C)
    try:
        ctx.check(_abi.lib().cp_composite_device(ctx.handle, ct.byref(st), ct.byref(p), out,
                                                 blend, None, None, None), "composite")
        ctx.synchronize()
        rows = [0, 1, ch // 3, ch // 2, ch // 2 + 1, 2 * ch // 3, ch - 2, ch - 1]
        # frame i's output row y is its source row y + oy_i, columns ox_i .. ox_i + cw
        band = np.stack([
            frames[i, torch.as_tensor([y + int(origins[i, 1]) for y in rows], device=frames.device),
                   int(origins[i, 0]):int(origins[i, 0]) + cw].cpu().numpy() for i in range(n)])
        ref = oracle.composite(band, p, threads=8)
        got_o = np.stack([ctx.download(out + y * cw * C, (cw, C)) for y in rows])
        got_b = np.stack([ctx.download(blend + y * cw * C, (cw, C)) for y in rows])
        cases.assert_close_u8(got_o, ref[0], what="cropped composite")
        cases.assert_close_u8(got_b, ref[1], what="cropped blend mask")
    finally:
        ctx.free(out)
        ctx.free(blend)
        del frames
        torch.cuda.empty_cache()
