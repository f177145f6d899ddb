"""The launch autotuner of the single-stack outlier kernel (needs a GB300).

Every candidate configuration (phase A by word column or by pixel, one or two staging
buffers, CTAs per SM) must give the oracle's results, and a tuned launch must too; the
chosen configurations are reported and cached in a file that a new context reads."""
import ctypes as ct
import json
import os

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

SETTINGS = [dict(threshold="abs/0.05/0.2", outlier="extreme", background="first"),
            dict(threshold="abs/0.04/0.3", outlier="average", background="median"),
            dict(threshold="rel/2/4", outlier="forward", background="first"),
            dict(threshold="rel/2/4", outlier="last", background="random", seed=5)]


def report(ctx):
    buf = ct.create_string_buffer(1 << 16)
    assert _abi.lib().cp_ctx_tuning_report(ctx.handle, buf, len(buf)) == _abi.CP_OK
    return json.loads(buf.value.decode())


@pytest.mark.parametrize("n", [20, 50, 100])
@pytest.mark.parametrize("config", ["0,0,0", "2,0,0", "0,1,0", "2,1,0", "0,0,2", "2,0,1"])
def test_every_configuration_matches_oracle(ctx, n, config, monkeypatch):
    monkeypatch.setenv("CP_PX_CONFIG", config)
    rng = np.random.default_rng(n)
    frames = cases.random_stack(rng, n, 21, 70, 3, n_spots=5)
    for kw in SETTINGS:
        p = cases.params(mode="outlier", **kw)
        got = ctx.composite(frames, p, debug=True)
        ref = oracle.composite(frames, p, debug=True)
        cases.assert_close_u8(got[0], ref[0], what="%s %s composite" % (config, kw))
        cases.assert_close_u8(got[1], ref[1], what="%s %s blend" % (config, kw))
        assert got[2] == ref[2]
        for k in ("median", "outlier_bits", "chosen", "background", "n_outliers"):
            assert np.array_equal(got[3][k], ref[3][k]), k


def device_composite(c, frames, p):
    """cp_composite_device on a device-resident stack: one launch over the whole frame (the
    host-memory entry point launches per row band, each too small to be tuned)."""
    n, h, w, ch = frames.shape
    lib = _abi.lib()
    base = c.upload(frames)
    out, blend = c.alloc(h * w * ch), c.alloc(h * w * ch)
    try:
        st = _abi.Stack(n=n, width=w, height=h, channels=ch, base=base, frame_stride=h * w * ch)
        c.check(lib.cp_composite_device(c.handle, ct.byref(st), ct.byref(p), out, blend, None,
                                        None, None), "cp_composite_device")
        c.synchronize()
        return (c.download(out, (h, w, ch)), c.download(blend, (h, w, ch)))
    finally:
        for ptr in (base, out, blend):
            c.free(ptr)


def test_tuned_launch_matches_oracle_and_is_cached(tmp_path, monkeypatch):
    """A stack large enough to tune (over 8 tiles of 128 pixels per SM): the tuned launch
    equals the oracle, the report names the key, and a second context reads the choice from
    the cache file instead of measuring again."""
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("CP_TUNE_CACHE", str(cache))
    monkeypatch.delenv("CP_AUTOTUNE", raising=False)
    monkeypatch.delenv("CP_PX_CONFIG", raising=False)
    rng = np.random.default_rng(77)
    frames = cases.random_stack(rng, 40, 480, 640, 3, n_spots=20)
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="average",
                     background="first")
    ref = oracle.composite(frames, p, threads=8)
    with cg.Context(0) as c1:
        got = device_composite(c1, frames, p)
        rep = report(c1)
    cases.assert_close_u8(got[0], ref[0], what="tuned composite")
    cases.assert_close_u8(got[1], ref[1], what="tuned blend")
    assert len(rep) == 1 and rep[0]["from"] == "measured", rep
    assert rep[0]["tuned_ms"] <= rep[0]["static_ms"] + 1e-6
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and json.loads(lines[0])["name"] == rep[0]["key"]
    with cg.Context(0) as c2:
        got2 = device_composite(c2, frames, p)
        rep2 = report(c2)
        # the host-memory entry point's band launches use the cached choice too
        got3 = c2.composite(frames, p)
    assert np.array_equal(got2[0], got[0]) and np.array_equal(got3[0], got[0])
    assert rep2[0]["from"] == "cache" and len(cache.read_text().strip().splitlines()) == 1


def test_autotune_off_and_small_stacks_are_not_tuned(tmp_path, monkeypatch):
    """CP_AUTOTUNE=0 launches the static choice without measuring; a stack under the size
    threshold is not tuned either. Neither writes the cache."""
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("CP_TUNE_CACHE", str(cache))
    monkeypatch.delenv("CP_PX_CONFIG", raising=False)
    rng = np.random.default_rng(78)
    big = cases.random_stack(rng, 24, 480, 640, 3, n_spots=10)
    small = cases.random_stack(rng, 24, 40, 64, 3, n_spots=3)
    p = cases.params(mode="outlier", threshold="rel/2/4", outlier="forward", background="first")
    with cg.Context(0) as c:
        monkeypatch.setenv("CP_AUTOTUNE", "0")
        got = device_composite(c, big, p)
        monkeypatch.delenv("CP_AUTOTUNE")
        got_small = device_composite(c, small, p)
        assert report(c) == []
    assert not cache.exists() or cache.read_text() == ""
    cases.assert_close_u8(got[0], oracle.composite(big, p, threads=8)[0], what="static")
    cases.assert_close_u8(got_small[0], oracle.composite(small, p)[0], what="small")
