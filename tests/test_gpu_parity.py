"""CUDA kernels against the oracle through the C ABI (needs a GB300).

Bit-exact: median, quartiles, outlier flags, chosen index, background index, outlier count
and warnings. Composite and blend mask: within 1 LSB per band (the benchmark spec's tolerance);
the kernels reproduce the reference's f32 operation order, so the error is expected to be 0
and the max/mean error is reported."""
import ctypes as ct

import numpy as np
import pytest

from chrono_photo_gb300 import _abi, example_data
from chrono_photo_gb300 import api as cg_api
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

OUTLIERS = ["first", "last", "extreme", "average", "forward", "backward"]
BACKGROUNDS = ["first", "random", "average", "median"]


def compare(ctx, frames, offset=0, crop=None, out_size=None, **kw):
    p = cases.params(**kw)
    ref = oracle.composite(frames, p, frame_offset=offset, crop=crop, out_size=out_size,
                           debug=kw.get("mode", "outlier") == "outlier", threads=8)
    if crop is not None:
        got = ctx.composite(frames, p, frame_offset=offset, crop=(crop, out_size),
                            debug=kw.get("mode", "outlier") == "outlier")
    else:
        got = ctx.composite(frames, p, frame_offset=offset,
                            debug=kw.get("mode", "outlier") == "outlier")
    err = cases.assert_close_u8(got[0], ref[0], what="composite")
    if kw.get("mode", "outlier") == "outlier":
        cases.assert_close_u8(got[1], ref[1], what="blend mask")
        assert got[2] == ref[2], "warnings"
        g, r = got[3], ref[3]
        for k in ("median", "outlier_bits", "chosen", "background", "n_outliers"):
            assert np.array_equal(g[k], r[k]), k
        if not p.thr_abs:
            assert np.array_equal(g["q1"], r["q1"]) and np.array_equal(g["q3"], r["q3"])
    return err


@pytest.mark.parametrize("case", cases.kat()["pixels"], ids=lambda c: c["name"])
def test_pixel_kat_gpu(ctx, case):
    st = cases.pixel_stack(case["samples"])
    p = cases.params(mode="outlier", threshold=case["threshold"], outlier=case["outlier"],
                     background=case["background"], weights=case["weights"], fade=case.get("fade"))
    out, blend, warn = ctx.composite(st, p)
    assert out.reshape(-1).tolist() == case["expect_pixel"]
    assert blend.reshape(-1)[0] == case["expect_mask"]


@pytest.mark.parametrize("case", cases.kat()["simple"], ids=lambda c: c["name"])
def test_simple_kat_gpu(ctx, case):
    st = cases.pixel_stack(case["samples"])
    p = cases.params(mode="darker" if case["darker"] else "lighter", weights=case["weights"],
                     fade=case.get("fade"))
    assert ctx.composite(st, p, blend=False)[0].reshape(-1).tolist() == case["expect_pixel"]


@pytest.fixture(scope="module")
def small():
    """16 frames of 640x480 with a moving r=20 disk (seed 1), at half size for speed."""
    return example_data.small_stack(seed=1, scale=2)


@pytest.fixture(scope="module")
def small_full():
    """The small-stack configuration at its stated size: 16 frames of 640x480 (seed 1)."""
    return example_data.small_stack(seed=1, scale=1)


@pytest.mark.parametrize("kw", [
    dict(threshold="abs/0.05/0.2", outlier="extreme", background="first"),
    dict(threshold="abs/0.05/0.2", outlier="extreme", background="random", seed=3),
    dict(threshold="abs/0.05/0.2", outlier="average", background="average"),
    dict(threshold="rel/3/6", outlier="forward", background="median")],
    ids=["extreme-first", "extreme-random", "average-average", "rel-forward-median"])
def test_config1_full_size(ctx, small_full, kw):
    """16 x 640x480, abs/0.05/0.2 extreme (the configuration's own settings) and three other
    settings, against the oracle on the whole frame: every debug output bit-exact."""
    compare(ctx, small_full, mode="outlier", **kw)


@pytest.mark.parametrize("outlier", OUTLIERS)
def test_small_stack_outlier_modes(ctx, small, outlier):
    compare(ctx, small, mode="outlier", threshold="abs/0.05/0.2", outlier=outlier,
            background="first")


@pytest.mark.parametrize("background", BACKGROUNDS)
def test_small_stack_backgrounds(ctx, small, background):
    compare(ctx, small, mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
            background=background, seed=99)


@pytest.mark.parametrize("outlier", ["average", "forward", "backward", "extreme"])
def test_rel_threshold(ctx, small, outlier):
    compare(ctx, small, mode="outlier", threshold="rel/3/6", outlier=outlier, background="first")


@pytest.mark.parametrize("mode", ["darker", "lighter"])
def test_simple(ctx, small, mode):
    compare(ctx, small, mode=mode)
    compare(ctx, small, mode=mode, weights=[0.3, 0.59, 0.11, 1], fade="clamp/abs/0,0/8,1")


@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 8, 16, 31, 32, 33, 63, 64, 65, 100, 127, 128])
def test_frame_counts(ctx, n):
    rng = np.random.default_rng(n)
    frames = cases.random_stack(rng, n, 13, 37, 3, n_spots=6)
    compare(ctx, frames, mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
            background="first")
    compare(ctx, frames, mode="outlier", threshold="abs/0.03/0.1", outlier="forward",
            background="average")
    if n >= 3:
        compare(ctx, frames, mode="outlier", threshold="rel/2/4", outlier="average",
                background="median")


@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("n", [33, 48, 64])
def test_rel_33_to_64_frames(ctx, n, c):
    """Rel thresholds on 33..64 frames: the radix selections over two 32-frame plane words
    give quartiles, medians and their successors for every channel count, with weights and
    a subsample (the sample mask is the selections' initial candidate set)."""
    rng = np.random.default_rng(300 + n * 10 + c)
    frames = cases.random_stack(rng, n, 11, 45, c, n_spots=5)
    compare(ctx, frames, mode="outlier", threshold="rel/2/4", outlier="extreme",
            background="first")
    compare(ctx, frames, mode="outlier", threshold="rel/1/3", outlier="average",
            background="median", weights=[0.5, 1, 2, 1])
    compare(ctx, frames, mode="outlier", threshold="rel/1.5/3", outlier="backward",
            background="first", sample=list(range(0, n, 2)))
    compare(ctx, frames, mode="outlier", threshold="rel/1.5/3", outlier="first",
            background="average", sample=list(range(1, n, 3)))


@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (17, 29), (64, 64), (33, 300)])
def test_shapes_channels(ctx, c, shape):
    rng = np.random.default_rng(c * 100 + shape[0])
    frames = cases.random_stack(rng, 12, shape[0], shape[1], c)
    compare(ctx, frames, mode="outlier", threshold="abs/0.05/0.2", outlier="last",
            background="first", weights=[1, 1, 1, 0])
    compare(ctx, frames, mode="lighter")


@pytest.mark.parametrize("weights", [[1, 1, 0, 1], [0.5, 1, 2, 1], [1, -1, 1, 1], [0, 0, 1, 1]])
def test_weights(ctx, weights):
    rng = np.random.default_rng(5)
    frames = cases.random_stack(rng, 20, 31, 41, 3)
    compare(ctx, frames, mode="outlier", threshold="abs/0.05/0.2", outlier="forward",
            background="median", weights=weights)
    compare(ctx, frames, mode="outlier", threshold="rel/1.5/3", outlier="extreme",
            background="average", weights=weights)


@pytest.mark.parametrize("fade_s,offset", [("clamp/abs/0,0/10,1", 0), ("repeat/abs/2,1/5,0.25", 7),
                                           ("clamp/rel/0,1/4,0", 0)])
def test_fades(ctx, fade_s, offset):
    rng = np.random.default_rng(9)
    frames = cases.random_stack(rng, 14, 20, 30, 3)
    for outlier in ("backward", "average", "extreme"):
        compare(ctx, frames, offset=offset, mode="outlier", threshold="abs/0.04/0.3",
                outlier=outlier, background="first", fade=fade_s)


def test_sample_subset(ctx):
    rng = np.random.default_rng(12)
    frames = cases.random_stack(rng, 40, 20, 30, 3)
    compare(ctx, frames, mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
            background="first", sample=[0, 3, 4, 8, 11, 20, 33, 39])
    compare(ctx, frames, mode="outlier", threshold="rel/3/6", outlier="last",
            background="median", sample=list(range(1, 40, 3)))


@pytest.mark.parametrize("thr", ["abs/0/0.1", "abs/1/1", "abs/0.02", "rel/0/1", "rel/0.5",
                                 "abs/30/40"])
def test_threshold_edges(ctx, thr):
    rng = np.random.default_rng(21)
    frames = cases.random_stack(rng, 9, 16, 16, 3)
    compare(ctx, frames, mode="outlier", threshold=thr, outlier="extreme", background="first")
    compare(ctx, frames, mode="outlier", threshold=thr, outlier="forward", background="random")


def test_crop_offsets(ctx):
    """Shake-corrected stacks: per-frame crop origins applied as address offsets."""
    rng = np.random.default_rng(4)
    frames = cases.random_stack(rng, 10, 40, 300, 3)
    offs = np.array([[0, 0], [3, -2], [-1, 4], [5, 1], [-7, -3], [2, 2], [0, 6], [1, -1],
                     [4, 0], [-2, 5]])
    crops = oracle.crop_create(offs, 300, 40)
    origins = crops[:, :2]
    size = (int(crops[0, 2]), int(crops[0, 3]))
    compare(ctx, frames, crop=origins, out_size=size, mode="outlier", threshold="abs/0.05/0.2",
            outlier="extreme", background="first")
    compare(ctx, frames, crop=origins, out_size=size, mode="darker")


def test_device_entry_point_matches_host(ctx, small):
    """cp_composite_device on device-resident frames equals the host-staged cp_composite."""
    n, h, w, c = small.shape
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="average",
                     background="average")
    ref = ctx.composite(small, p)
    fb = ctx.upload(small)
    out = ctx.alloc(h * w * c)
    bl = ctx.alloc(h * w * c)
    warn = ctx.alloc(8)
    ctx.upload(np.zeros(1, np.uint64), warn)
    try:
        st = _abi.Stack(n=n, width=w, height=h, channels=c, base=fb, frame_stride=h * w * c)
        rc = _abi.lib().cp_composite_device(ctx.handle, ct.byref(st), ct.byref(p), out, bl,
                                            None, warn, None)
        ctx.check(rc)
        ctx.synchronize()
        assert np.array_equal(ctx.download(out, (h, w, c)), ref[0])
        assert np.array_equal(ctx.download(bl, (h, w, c)), ref[1])
        assert int(ctx.download(warn, (1,), np.uint64)[0]) == ref[2]
    finally:
        for q in (fb, out, bl, warn):
            ctx.free(q)


MULTI_SETTINGS = [
    dict(mode="outlier", threshold="abs/0.05/0.2", outlier="average", background="first"),
    dict(mode="outlier", threshold="rel/3/6", outlier="extreme", background="random"),
    dict(mode="darker"),
    dict(mode="outlier", threshold="abs/0.1/0.3", outlier="forward", background="average",
         fade="clamp/rel/0,0.2/8,1"),
    dict(mode="lighter", weights=[0.3, 0.6, 0.1, 1]),
    dict(mode="outlier", threshold="abs/0.02", outlier="backward", background="median",
         sample=[0, 2, 4, 6, 8, 10, 12, 14]),
]


def test_composite_multi_matches_single_calls(ctx, small):
    """cp_composite_multi (one upload, several settings) gives each setting exactly what
    cp_composite gives it alone, warnings included."""
    ps = [cases.params(**kw) for kw in MULTI_SETTINGS]
    got = ctx.composite_multi(small, ps)
    for p, (o, b, wn) in zip(ps, got):
        ref = ctx.composite(small, p)
        assert np.array_equal(o, ref[0])
        assert (b is None and ref[1] is None) or np.array_equal(b, ref[1])
        assert wn == ref[2]
        oref = oracle.composite(small, p, threads=8)
        cases.assert_close_u8(o, oref[0], what="composite")


def test_composite_multi_limits(ctx, small):
    p = cases.params()
    with pytest.raises(_abi.ChronoError) as e:
        ctx.composite_multi(small, [p] * (_abi.CP_MAX_SETTINGS + 1))
    assert e.value.status == _abi.CP_ERR_LIMIT
    with pytest.raises(_abi.ChronoError) as e:
        ctx.composite_multi(small, [])
    assert e.value.status == _abi.CP_ERR_ARG
    assert len(ctx.composite_multi(small, [p] * _abi.CP_MAX_SETTINGS)) == _abi.CP_MAX_SETTINGS


def test_invalid_stacks(ctx):
    f = np.zeros((129, 2, 2, 3), np.uint8)
    with pytest.raises(_abi.ChronoError) as e:
        ctx.composite(f, cases.params())
    assert e.value.status == _abi.CP_ERR_ARG
    with pytest.raises(_abi.ChronoError):
        ctx.composite(np.zeros((2, 2, 2, 3), np.uint8), cases.params(threshold="rel/1/2"))
    with pytest.raises(_abi.ChronoError):
        ctx.composite(np.zeros((4, 2, 2, 2), np.uint8), cases.params())


def test_processors_take_png_paths(ctx, small, tmp_path):
    """OutlierProcessor / SimpleProcessor on PNG file paths (decoded by cp_load_png, only the
    selected frames) equal the same calls on the arrays."""
    paths = example_data.write_pngs(small, str(tmp_path), level=1, threads=4)
    sel = list(range(3, 15))
    op = cg_api.OutlierProcessor(threshold="abs/0.05/0.2", background="first",
                                 outlier="forward", fade="clamp/abs/0,0.3/10,1", context=ctx)
    a = op.process(small, image_indices=sel)
    b = op.process(paths, image_indices=sel)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    sp = cg_api.SimpleProcessor(darker=False, context=ctx)
    assert np.array_equal(sp.process(small), sp.process(paths))


@pytest.mark.parametrize("thr,weights", [("rel/3/6", [1, 0, 1, 1]), ("rel/2/5", [0.5, 2.0, 0, 1]),
                                         ("abs/0.05/0.2", [0.5, 0, 2.0, 1])])
def test_paired_distances_with_a_weight_zero_channel(ctx, thr, weights):
    """Paired-f32 distances (rel thresholds, or abs with weights other than 0/1) where one
    channel has weight 0: that channel adds +0 to every distance, as the reference's skipped
    term does (src/chrono.rs:261-279), including a word of 32 samples and a partial one."""
    rng = np.random.default_rng(31)
    frames = cases.random_stack(rng, 45, 16, 48, 3, n_spots=6)
    for outlier in ("extreme", "average", "forward"):
        compare(ctx, frames, mode="outlier", threshold=thr, outlier=outlier, background="first",
                weights=weights)
