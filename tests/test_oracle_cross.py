"""The C++ oracle against the independent pure-Python restatement on random small stacks
(CPU only): every outlier/background mode, abs and rel thresholds, weights, fades and
median subsamples. Two restatements written separately agreeing bit for bit is what pins
the oracle beyond the known answers."""
import itertools

import numpy as np
import pytest

from chrono_photo_gb300.api import Fade, Threshold
from oracle import oracle, pyref
from tests import cases

OUTLIERS = ["first", "last", "extreme", "average", "forward", "backward"]
BACKGROUNDS = ["first", "random", "average", "median"]


def _check_stack(frames, thr_s, outlier, background, weights, fade_s=None, sample=None,
                 offset=0, seed=11):
    p = cases.params(mode="outlier", threshold=thr_s, outlier=outlier, background=background,
                     weights=weights, fade=fade_s, sample=sample, seed=seed)
    out, blend, warn, dbg = oracle.composite(frames, p, frame_offset=offset, debug=True)
    thr = Threshold.parse(thr_s)
    t = pyref.Threshold(thr.absolute, thr.min, thr.max)
    fd = Fade.parse(fade_s) if fade_s else Fade.none()
    fade = pyref.fade_table(fd.repeat, fd.absolute, fd.points)
    n, h, w, c = frames.shape
    lib = oracle.lib()
    nwarn = 0
    for y in range(h):
        for x in range(w):
            pid = y * w + x
            samples = [tuple(int(v) for v in frames[i, y, x]) for i in range(n)]
            pix, mask, wn, det = pyref.calc_pixel(
                samples, t, weights, background, outlier, fade, offset, sample_idx=sample,
                rng=lambda m, pid=pid: lib.or_gen_range(seed, pid, m))
            nwarn += wn
            assert tuple(out[y, x].tolist()) == pix, (y, x)
            assert blend[y, x, 0] == mask, (y, x)
            bits = dbg["outlier_bits"][y, x]
            got = [i for i in range(n) if (int(bits[i // 32]) >> (i % 32)) & 1]
            assert got == det["outliers"], (y, x)
            assert np.array_equal(dbg["median"][y, x], np.asarray(det["median"], np.float32))
            assert dbg["chosen"][y, x] == det["chosen"]
            assert dbg["background"][y, x] == det["background"]
    assert warn == nwarn


@pytest.mark.parametrize("outlier,background", list(itertools.product(OUTLIERS, BACKGROUNDS)))
def test_modes_abs(outlier, background):
    rng = np.random.default_rng(hash((outlier, background)) % 2 ** 32)
    frames = cases.random_stack(rng, 9, 5, 6, 3)
    _check_stack(frames, "abs/0.05/0.2", outlier, background, [1, 1, 1, 1])


@pytest.mark.parametrize("outlier", OUTLIERS)
def test_modes_rel(outlier):
    rng = np.random.default_rng(100 + OUTLIERS.index(outlier))
    frames = cases.random_stack(rng, 8, 5, 5, 3)
    _check_stack(frames, "rel/3/6", outlier, "first", [1, 1, 1, 1])


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 16, 33])
def test_frame_counts(n):
    rng = np.random.default_rng(n)
    frames = cases.random_stack(rng, n, 4, 5, 3)
    _check_stack(frames, "abs/0.05/0.2", "extreme", "first", [1, 1, 1, 1])
    if n >= 3:
        _check_stack(frames, "rel/2/4", "average", "average", [1, 1, 1, 1])


@pytest.mark.parametrize("weights", [[1, 1, 0, 1], [0.5, 1, 2, 1], [1, -1, 1, 1], [0, 0, 1, 1]])
def test_weights(weights):
    rng = np.random.default_rng(5)
    frames = cases.random_stack(rng, 9, 4, 5, 3)
    _check_stack(frames, "abs/0.05/0.2", "forward", "median", weights)
    _check_stack(frames, "rel/1.5/3", "extreme", "average", weights)


@pytest.mark.parametrize("fade_s,offset", [("clamp/abs/0,0/10,1", 0), ("repeat/abs/2,1/5,0.25", 7),
                                           ("clamp/rel/0,1/4,0", 0), ("repeat/rel/0,0.2/3,1/6,0", 3)])
def test_fades(fade_s, offset):
    rng = np.random.default_rng(9)
    frames = cases.random_stack(rng, 9, 4, 4, 3)
    _check_stack(frames, "abs/0.04/0.3", "backward", "first", [1, 1, 1, 1], fade_s, offset=offset)
    _check_stack(frames, "abs/0.04/0.3", "average", "first", [1, 1, 1, 1], fade_s, offset=offset)


def test_sample_subset():
    rng = np.random.default_rng(12)
    frames = cases.random_stack(rng, 12, 4, 5, 3)
    _check_stack(frames, "abs/0.05/0.2", "extreme", "first", [1, 1, 1, 1], sample=[0, 3, 4, 8, 11])
    _check_stack(frames, "rel/3/6", "last", "median", [1, 1, 1, 1], sample=[1, 2, 5, 6, 7, 9])


@pytest.mark.parametrize("thr", ["abs/0/0.1", "abs/1/1", "abs/0.02", "rel/0/1", "rel/0.5"])
def test_threshold_edges(thr):
    rng = np.random.default_rng(21)
    frames = cases.random_stack(rng, 6, 4, 4, 3)
    _check_stack(frames, thr, "extreme", "first", [1, 1, 1, 1])
    _check_stack(frames, thr, "forward", "random", [1, 1, 1, 1])


@pytest.mark.parametrize("c", [1, 4])
def test_channels(c):
    rng = np.random.default_rng(30 + c)
    frames = cases.random_stack(rng, 7, 4, 5, c)
    _check_stack(frames, "abs/0.05/0.2", "extreme", "average", [1, 1, 1, 0])


def test_simple_modes():
    rng = np.random.default_rng(3)
    frames = cases.random_stack(rng, 9, 5, 6, 3)
    for darker in (True, False):
        for weights, fade_s in [([1, 1, 1, 1], None), ([0.3, 0.59, 0.11, 1], "clamp/abs/0,0/8,1")]:
            p = cases.params(mode="darker" if darker else "lighter", weights=weights, fade=fade_s)
            out, _, _ = oracle.composite(frames, p)
            fd = Fade.parse(fade_s) if fade_s else Fade.none()
            fade = pyref.fade_table(fd.repeat, fd.absolute, fd.points)
            for y in range(frames.shape[1]):
                for x in range(frames.shape[2]):
                    samples = [tuple(int(v) for v in frames[i, y, x]) for i in range(frames.shape[0])]
                    assert tuple(out[y, x].tolist()) == pyref.simple_pixel(samples, weights, darker, fade, 0)
