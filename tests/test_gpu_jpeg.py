"""JPEG frame ingest on the GPU (needs a GB300): nvJPEG's decoding held to the oracle's
exact-IDCT decoder with the tolerances below; the processors take .jpg paths end to end (frames decoded into device memory,
composited there) with the composite of the same decoded frames; batches over the 64-file
decode batch and mixed engine / software routes; header errors reported per file, the
context usable afterwards."""
import os

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

ROUTES = [("engine", None), ("software", "default"), ("gpu-hybrid", "gpu")]
# Tolerance per route: (largest difference in RGB, in gray, largest mean difference). A
# decoder whose inverse DCT is off by 1 in a Y, Cb or Cr sample moves R, G and B by up to
# 1 + 1.772 levels after conversion, so 3 in RGB is the bound of a one-level IDCT error;
# measured on a GB300 over 100 random-colour cases (q 50-100, 4:4:4 and 4:2:0, up to
# 640x480): engines 3 / 1 / 0.059, software backends 2 / 1 / 0.0001.
TOLERANCE = {"engine": (3, 1, 0.1), "software": (2, 1, 0.01), "gpu-hybrid": (2, 1, 0.01)}


def assert_near_oracle(got, ref, route):
    d = np.abs(got.astype(int) - ref.astype(int))
    rgb, gray, mean = TOLERANCE[route]
    assert d.max() <= (gray if got.shape[-1] == 1 else rgb) and d.mean() < mean, \
        (route, int(d.max()), d.mean())


def write_stack(tmp_path, frames, quality=95, subsampling="444", prefix="f"):
    paths = []
    for i, f in enumerate(frames):
        p = tmp_path / ("%s%04d.jpg" % (prefix, i))
        cg.save_jpeg(p, f, quality=quality, subsampling=subsampling)
        paths.append(str(p))
    return paths


def oracle_stack(paths):
    return np.stack([oracle.jpeg_decode(open(p, "rb").read()) for p in paths])


@pytest.fixture
def route_ctx(request, monkeypatch):
    name, env = request.param
    if env:
        monkeypatch.setenv("CP_JPEG_BACKEND", env)
    else:
        monkeypatch.delenv("CP_JPEG_BACKEND", raising=False)
    with cg.Context(0) as c:  # the route is fixed at the context's first decode
        c.route = name
        yield c


@pytest.mark.parametrize("route_ctx", ROUTES, ids=[r[0] for r in ROUTES], indirect=True)
@pytest.mark.parametrize("h,w,c,q,ss", [(48, 64, 3, 95, "444"), (37, 53, 3, 75, "444"),
                                        (41, 29, 3, 60, "420"), (120, 200, 3, 90, "420"),
                                        (40, 56, 1, 95, "444"), (480, 640, 3, 95, "444")])
def test_decode_within_one_level_of_oracle(tmp_path, route_ctx, h, w, c, q, ss):
    rng = np.random.default_rng(h * w)
    frames = cases.random_stack(rng, 3, h, w, 3, n_spots=2)
    if c == 1:
        frames = frames[..., :1].copy()
    paths = write_stack(tmp_path, frames, q, ss)
    ref = oracle_stack(paths)
    got = cg.load_jpeg(paths, context=route_ctx)
    assert got.shape == ref.shape
    assert_near_oracle(got, ref, route_ctx.route)
    dev, stride, shape = route_ctx.load_jpeg_device(paths)
    try:
        raw = route_ctx.download(dev, (shape[0] * stride,))
    finally:
        route_ctx.free(dev)
    fb = h * w * c
    dgot = np.stack([raw[i * stride:i * stride + fb].reshape(h, w, c) for i in range(shape[0])])
    assert np.array_equal(dgot, got)


def test_many_files_and_mixed_routes(tmp_path, ctx):
    """70 files (two decode batches); every third rewritten as extended-sequential (SOF1),
    a stream the JPEG engines do not take, so one call mixes both routes."""
    rng = np.random.default_rng(9)
    frames = cases.random_stack(rng, 70, 24, 40, 3, n_spots=3)
    paths = write_stack(tmp_path, frames, 92, "420")
    for p in paths[::3]:
        d = bytearray(open(p, "rb").read())
        sof = d.index(b"\xff\xc0")
        d[sof + 1] = 0xC1
        open(p, "wb").write(bytes(d))
    assert_near_oracle(cg.load_jpeg(paths, context=ctx), oracle_stack(paths), "engine")


@pytest.mark.parametrize("mode", ["outlier", "darker"])
def test_processors_take_jpeg_paths(tmp_path, ctx, mode):
    """OutlierProcessor / SimpleProcessor .process(jpg paths): frames decoded into device
    memory and composited there, equal to the composite of the same decoded frames from
    host memory, which matches the oracle's composite of them."""
    rng = np.random.default_rng(3)
    frames = cases.random_stack(rng, 20, 60, 80, 3, n_spots=4)
    paths = write_stack(tmp_path, frames)
    dec = cg.load_jpeg(paths, context=ctx)
    if mode == "outlier":
        proc = cg.OutlierProcessor(threshold=cg.Threshold.abs(0.05, 0.2), background="first",
                                   outlier="extreme", context=ctx)
        out, blend = proc.process(paths)
        ref = ctx.composite(dec, mode="outlier", threshold="abs/0.05/0.2", background="first",
                            outlier="extreme")
        assert np.array_equal(out, ref[0]) and np.array_equal(blend, ref[1])
        o = oracle.composite(dec, cases.params(mode="outlier", threshold="abs/0.05/0.2",
                                               background="first", outlier="extreme"))
        cases.assert_close_u8(out, o[0], what="jpeg outlier composite")
        # a window of the files, as chrono-video selects them: the frame offset follows
        out2, _ = proc.process(paths, image_indices=list(range(5, 15)))
        ref2 = ctx.composite(dec[5:15], mode="outlier", threshold="abs/0.05/0.2",
                             background="first", outlier="extreme", frame_offset=5)
        assert np.array_equal(out2, ref2[0])
    else:
        out = cg.SimpleProcessor(darker=True, context=ctx).process(paths)
        ref = ctx.composite(dec, mode="darker", blend=False)[0]
        assert np.array_equal(out, ref)


def test_errors_per_file_and_context_recovers(tmp_path, ctx):
    rng = np.random.default_rng(4)
    frames = cases.random_stack(rng, 4, 32, 48, 3, n_spots=2)
    paths = write_stack(tmp_path, frames)
    other = str(tmp_path / "other.jpg")
    cg.save_jpeg(other, frames[0][:16])  # another height
    lib = _abi.lib()
    for bad, what in ((paths[:2] + [other] + paths[2:], "other.jpg"),
                      (paths[:3] + [str(tmp_path / "missing.jpg")], "missing.jpg")):
        with pytest.raises(cg.ChronoError) as e:
            cg.load_jpeg(bad, context=ctx)
        assert e.value.status == _abi.CP_ERR_IO and what in str(e.value)
    gray = str(tmp_path / "gray.jpg")
    cg.save_jpeg(gray, frames[0][..., :1])
    with pytest.raises(cg.ChronoError):  # one component where three are asked for
        cg.load_jpeg(paths[:1] + [gray], context=ctx)
    ptr = ctx.alloc(64)
    try:
        arr = (_abi.ct.c_char_p * 1)(paths[0].encode())
        assert lib.cp_load_jpeg_device(ctx.handle, arr, 1, 0, ptr, 16, 48, 32, 3) == \
            _abi.CP_ERR_ARG  # frame stride below one frame
    finally:
        ctx.free(ptr)
    assert_near_oracle(cg.load_jpeg(paths, context=ctx), oracle_stack(paths), "engine")
