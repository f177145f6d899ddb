"""Several settings of one stack in one pass (needs a GB300): cp_composite_device_multi and
cp_composite_multi give every setting exactly what cp_composite_device gives it alone
(composite, blend mask and warnings), whatever the mix: settings sharing their distance pass,
abs and rel thresholds together (quartiles), every outlier mode and background, weights,
fades, a --sample shared by some settings only, darker / lighter (folded on the same staged
rows, integer and f32 forms), 1, 2 and 4 plane words, more settings than one multi-setting
launch holds; and the single-setting results match the oracle."""
import ctypes as ct

import numpy as np
import pytest

from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

OUTLIERS = ["first", "last", "extreme", "average", "forward", "backward"]
BACKGROUNDS = ["first", "random", "average", "median"]


def bench_six():
    return [dict(mode="outlier", threshold="abs/0.05/0.2", outlier=o, background="first")
            for o in ("average", "forward", "backward")] + [
        dict(mode="outlier", threshold="rel/3/6", outlier="average", background="first"),
        dict(mode="darker"), dict(mode="lighter")]


def mixed():
    s = []
    for i, o in enumerate(OUTLIERS):
        s.append(dict(mode="outlier", threshold="abs/0.05/0.2", outlier=o,
                      background=BACKGROUNDS[i % 4], seed=7 + i))
    s += [dict(mode="outlier", threshold="rel/2/4", outlier="forward", background="median"),
          dict(mode="outlier", threshold="rel/3/6", outlier="extreme", background="random"),
          dict(mode="outlier", threshold="abs/0.1/0.3", outlier="average", background="average",
               fade="clamp/rel/0,0.2/8,1"),
          dict(mode="outlier", threshold="abs/0.04", outlier="last", background="first",
               weights=[1, 0, 1, 1]),
          dict(mode="outlier", threshold="abs/0.05/0.2", outlier="backward", background="first",
               weights=[0.5, 2.0, 1.0, 1]),
          dict(mode="lighter"),
          dict(mode="darker", weights=[0.3, 0.59, 0.11, 1], fade="clamp/abs/0,0/8,1"),
          dict(mode="outlier", threshold="abs/0.02", outlier="extreme", background="median",
               sample=[0, 2, 4, 6, 8, 10, 12, 14])]
    return s


def device_multi(ctx, frames, ps):
    """cp_composite_device_multi on an uploaded stack whose frames start on 16-byte
    boundaries (the stacks the multi-setting kernel takes): [(composite, blend, warnings)]."""
    n, h, w, c = frames.shape
    lib = _abi.lib()
    fb = h * w * c
    stride = (fb + 15) // 16 * 16
    padded = np.zeros((n, stride), np.uint8)
    padded[:, :fb] = frames.reshape(n, fb)
    base = ctx.upload(padded)
    k = len(ps)
    outs = [ctx.alloc(fb) for _ in range(k)]
    blends = [ctx.alloc(fb) for _ in range(k)]
    warn = ctx.upload(np.zeros(k, np.uint64))
    try:
        st = _abi.Stack(n=n, width=w, height=h, channels=c, base=base, frame_stride=stride)
        arr = (_abi.Params * k)(*ps)
        o = (ct.c_void_p * k)(*outs)
        b = (ct.c_void_p * k)(*blends)
        ctx.check(lib.cp_composite_device_multi(ctx.handle, ct.byref(st), arr, k, o, b, warn, None),
                  "cp_composite_device_multi")
        ctx.synchronize()
        wn = ctx.download(warn, (k,), np.uint64)
        return [(ctx.download(outs[i], (h, w, c)), ctx.download(blends[i], (h, w, c)), int(wn[i]))
                for i in range(k)]
    finally:
        for ptr in [base, warn] + outs + blends:
            ctx.free(ptr)


def device_single(ctx, frames, p):
    return device_multi(ctx, frames, [p])[0]


@pytest.mark.parametrize("n", [20, 50, 100])
def test_device_multi_equals_single(ctx, n):
    rng = np.random.default_rng(n)
    frames = cases.random_stack(rng, n, 37, 90, 3, n_spots=5)
    kws = mixed()
    ps = [cases.params(**kw) for kw in kws]
    got = device_multi(ctx, frames, ps)
    for kw, p, (o, b, wn) in zip(kws, ps, got):
        ref = device_single(ctx, frames, p)
        assert np.array_equal(o, ref[0]), kw
        if kw["mode"] == "outlier":
            assert np.array_equal(b, ref[1]), kw
        assert wn == ref[2], kw


def test_bench_settings_match_oracle(ctx):
    """The benchmark's six settings in one call (three abs settings share one distance pass,
    rel/3/6 adds the quartiles), against the oracle."""
    rng = np.random.default_rng(11)
    frames = cases.random_stack(rng, 64, 48, 130, 3, n_spots=6)
    kws = bench_six()
    ps = [cases.params(**kw) for kw in kws]
    for kw, p, (o, b, wn) in zip(kws, ps, device_multi(ctx, frames, ps)):
        ref = oracle.composite(frames, p, threads=8)
        cases.assert_close_u8(o, ref[0], what="%s composite" % kw)
        if kw["mode"] == "outlier":
            cases.assert_close_u8(b, ref[1], what="%s blend" % kw)
            assert wn == ref[2]


def test_more_settings_than_one_launch(ctx):
    """12 outlier settings sharing their order statistics: two multi-setting launches."""
    rng = np.random.default_rng(12)
    frames = cases.random_stack(rng, 40, 33, 70, 3, n_spots=4)
    kws = [dict(mode="outlier", threshold=t, outlier=o, background="first")
           for t in ("abs/0.05/0.2", "rel/2/4") for o in OUTLIERS]
    ps = [cases.params(**kw) for kw in kws]
    got = device_multi(ctx, frames, ps)
    for kw, p, (o, b, wn) in zip(kws, ps, got):
        ref = device_single(ctx, frames, p)
        assert np.array_equal(o, ref[0]) and np.array_equal(b, ref[1]) and wn == ref[2], kw


def test_all_outliers_warnings_per_setting(ctx):
    """Pixels whose every frame is an outlier count a warning in the settings that see them
    (first background), each setting its own counter."""
    rng = np.random.default_rng(13)
    frames = rng.integers(0, 256, (9, 16, 32, 3), dtype=np.uint8)  # noise: many outliers
    kws = [dict(mode="outlier", threshold="abs/0.01", outlier=o, background="first")
           for o in ("extreme", "average", "forward")] + [
        dict(mode="outlier", threshold="abs/0.5", outlier="extreme", background="first")]
    ps = [cases.params(**kw) for kw in kws]
    got = device_multi(ctx, frames, ps)
    for p, (o, b, wn) in zip(ps, got):
        assert wn == oracle.composite(frames, p)[2]


def test_host_multi_equals_device_multi(ctx):
    rng = np.random.default_rng(14)
    frames = cases.random_stack(rng, 32, 41, 77, 3, n_spots=3)
    kws = bench_six()
    ps = [cases.params(**kw) for kw in kws]
    dev = device_multi(ctx, frames, ps)
    host = ctx.composite_multi(frames, ps)
    for kw, (o, b, wn), (ho, hb, hw) in zip(kws, dev, host):
        assert np.array_equal(o, ho) and wn == hw
        if kw["mode"] == "outlier":
            assert np.array_equal(b, hb)


def test_device_multi_arguments(ctx):
    lib = _abi.lib()
    frames = np.zeros((4, 8, 8, 3), np.uint8)
    p = cases.params()
    st = _abi.Stack(n=4, width=8, height=8, channels=3, base=None, frame_stride=192)
    arr = (_abi.Params * 1)(p)
    o = (ct.c_void_p * 1)(None)
    assert lib.cp_composite_device_multi(ctx.handle, ct.byref(st), arr, 1, o, None, None,
                                         None) == _abi.CP_ERR_ARG
    many = (_abi.Params * (_abi.CP_MAX_SETTINGS + 1))(*([p] * (_abi.CP_MAX_SETTINGS + 1)))
    om = (ct.c_void_p * (_abi.CP_MAX_SETTINGS + 1))()
    assert lib.cp_composite_device_multi(ctx.handle, ct.byref(st), many,
                                         _abi.CP_MAX_SETTINGS + 1, om, None, None,
                                         None) == _abi.CP_ERR_LIMIT
    del frames


def launch_counts(ctx):
    a, b, c = ct.c_uint64(), ct.c_uint64(), ct.c_uint64()
    ctx.check(_abi.lib().cp_ctx_launch_counts(ctx.handle, ct.byref(a), ct.byref(b), ct.byref(c)))
    return a.value, b.value, c.value


def test_benchmark_step_is_one_launch(ctx):
    """The benchmark's six settings (abs and rel thresholds, darker, lighter) of one aligned
    RGB stack take one multi-setting launch carrying all six; a setting with its own sample
    runs apart."""
    rng = np.random.default_rng(15)
    frames = cases.random_stack(rng, 64, 32, 64, 3, n_spots=3)
    ps = [cases.params(**kw) for kw in bench_six()]
    l0, m0, s0 = launch_counts(ctx)
    device_multi(ctx, frames, ps)
    l1, m1, s1 = launch_counts(ctx)
    assert (l1 - l0, m1 - m0, s1 - s0) == (1, 1, 6)
    other = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="first",
                         background="first", sample=list(range(0, 64, 2)))
    device_multi(ctx, frames, ps + [other])
    l2, m2, s2 = launch_counts(ctx)
    assert (l2 - l1, m2 - m1, s2 - s1) == (2, 1, 6)


@pytest.mark.parametrize("order", [("lighter", "darker"), ("darker", "lighter")])
def test_darker_lighter_pair(ctx, order):
    """Darker and lighter next to each other (0/1 weights, no fade) fold in one pass over the
    samples, whichever comes first; ties keep the earliest frame."""
    rng = np.random.default_rng(16)
    frames = cases.random_stack(rng, 40, 24, 48, 3, n_spots=3)
    frames[7] = frames[3]  # equal sums: the earlier frame wins
    kws = [dict(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                background="first")] + [dict(mode=m) for m in order]
    ps = [cases.params(**kw) for kw in kws]
    for kw, p, (o, b, wn) in zip(kws, ps, device_multi(ctx, frames, ps)):
        ref = device_single(ctx, frames, p)
        assert np.array_equal(o, ref[0]), kw
        cases.assert_close_u8(o, oracle.composite(frames, p)[0], what=str(kw))


def test_multi_paired_distances_with_a_weight_zero_channel(ctx):
    """Paired-f32 settings with a weight-0 channel in one multi-setting launch: each equals
    its single-setting result and the oracle."""
    rng = np.random.default_rng(41)
    frames = cases.random_stack(rng, 64, 24, 80, 3, n_spots=6)
    kws = [dict(mode="outlier", threshold="rel/3/6", outlier="extreme", background="first",
                weights=[1, 0, 1, 1]),
           dict(mode="outlier", threshold="abs/0.05/0.2", outlier="average", background="first",
                weights=[0.5, 0, 2.0, 1]),
           dict(mode="outlier", threshold="abs/0.05/0.2", outlier="forward", background="first",
                weights=[0.5, 0, 2.0, 1])]
    ps = [cases.params(**kw) for kw in kws]
    got = device_multi(ctx, frames, ps)
    for kw, p, (o, b, wn) in zip(kws, ps, got):
        ref = device_single(ctx, frames, p)
        assert np.array_equal(o, ref[0]) and np.array_equal(b, ref[1]) and wn == ref[2], kw
        orc = oracle.composite(frames, p)
        cases.assert_close_u8(o, orc[0], what="composite %s" % kw["threshold"])
        cases.assert_close_u8(b, orc[1], what="blend %s" % kw["threshold"])
        assert wn == orc[2]
