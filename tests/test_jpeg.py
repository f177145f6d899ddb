"""JPEG encode (cp_encode_jpeg / cp_save_jpeg) and the host half of JPEG ingest (headers,
errors), on the CPU, against the oracle's exact-IDCT decoder (oracle/jpeg_oracle.cpp).

Tolerances, stated once:
  - encoder: the oracle's decoding of a file is within the quantisation error of the
    source, bounded here by PSNR on noise-free ramps (>= 49 dB at quality 95 4:4:4,
    >= 45 dB at 95 4:2:0, >= 41 dB at 50 4:4:4, >= 42 dB at 90 for every size);
  - nvJPEG (the product's GPU decoder, golden decodings made on a GB300 by
    tests/golden/make_jpeg_golden.py): through the software backend within 1 level of the
    oracle in every gray sample and 2 levels in RGB (equal in the golden cases), through
    the GPU's JPEG engines within 3 levels in RGB and 1 in gray (their inverse DCT is off
    by up to 1 in a Y, Cb or Cr sample, which the colour conversion spreads to 1 + 1.772)
    with a mean absolute difference under 0.1.
"""
import os

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "jpeg_golden.npz")


def gradient(h, w, c=3):
    """Ramps of at most 3 levels per pixel (chroma subsampling keeps such an image)."""
    y, x = np.mgrid[0:h, 0:w]
    a = np.stack([np.minimum(255, 30 + 3 * x), np.minimum(255, 30 + 3 * y),
                  np.minimum(255, 120 + (x + y) // 2)], -1).astype(np.uint8)
    if c == 1:
        return a[..., :1]
    if c == 4:
        return np.concatenate([a, np.full((h, w, 1), 77, np.uint8)], -1)
    return a


def psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return 99.0 if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


@pytest.mark.parametrize("q,ss,floor", [(95, "444", 49), (95, "420", 45), (75, "444", 45),
                                        (50, "444", 41), (100, "444", 51)])
def test_round_trip_through_oracle(q, ss, floor):
    a = gradient(64, 96)
    d = oracle.jpeg_decode(cg.encode_jpeg(a, quality=q, subsampling=ss))
    assert d.shape == a.shape
    assert psnr(d, a) >= floor


@pytest.mark.parametrize("h,w,c", [(1, 1, 3), (7, 9, 3), (21, 37, 3), (8, 8, 1), (33, 70, 1),
                                   (17, 31, 4), (130, 3, 3)])
@pytest.mark.parametrize("ss", ["444", "420"])
def test_sizes_and_channels(h, w, c, ss):
    """Sizes off the 8 / 16 MCU grid, gray, and RGBA (alpha dropped, as image's encoder)."""
    a = gradient(h, w, c)
    data = cg.encode_jpeg(a, quality=90, subsampling=ss)
    d = oracle.jpeg_decode(data)
    ref = a[..., :3] if c == 4 else a
    assert d.shape == ref.shape
    assert psnr(d, ref) >= 42


def test_bytes_do_not_depend_on_threads():
    rng = np.random.default_rng(1)
    a = np.clip(gradient(200, 136).astype(int) + rng.normal(0, 6, (200, 136, 3)), 0,
                255).astype(np.uint8)
    ref = cg.encode_jpeg(a, quality=95, threads=1)
    for t in (2, 3, 16, 0):
        assert cg.encode_jpeg(a, quality=95, threads=t) == ref


def test_file_structure():
    """SOI, JFIF, 8-bit tables, SOF0 with the sampling asked for, DRI of one MCU row,
    interleaved SOS, EOI."""
    a = gradient(40, 50)
    for ss, luma in (("444", 0x11), ("420", 0x22)):
        d = cg.encode_jpeg(a, quality=95, subsampling=ss)
        assert d[:2] == b"\xff\xd8" and d[-2:] == b"\xff\xd9" and d[6:11] == b"JFIF\x00"
        sof = d.index(b"\xff\xc0")
        assert d[sof + 4] == 8 and d[sof + 5:sof + 7] == b"\x00\x28"  # height 40
        assert d[sof + 7:sof + 9] == b"\x00\x32" and d[sof + 9] == 3  # width 50, 3 comps
        assert d[sof + 11] == luma and d[sof + 14] == 0x11 and d[sof + 17] == 0x11
        dri = d.index(b"\xff\xdd")
        mcus_across = (50 + (8 if ss == "444" else 16) - 1) // (8 if ss == "444" else 16)
        assert d[dri + 4] * 256 + d[dri + 5] == mcus_across
        assert d.index(b"\xff\xda") > dri


def test_save_creates_parent_and_info(tmp_path):
    a = gradient(30, 44)
    p = tmp_path / "new_dir" / "out.jpg"
    cg.save_jpeg(p, a)
    assert cg.jpeg_info(p) == (44, 30, 3)
    assert psnr(oracle.jpeg_decode(p.read_bytes()), a) >= 48
    g = tmp_path / "gray.jpeg"
    cg.save_image(g, a[..., :1])
    assert cg.jpeg_info(g) == (44, 30, 1)
    cg.save_image(tmp_path / "x.png", a)
    assert cg.png_info(tmp_path / "x.png") == (44, 30, 3)


def test_encode_capacity_and_arguments():
    lib = _abi.lib()
    a = gradient(16, 16)
    size = _abi.ct.c_uint64(0)
    assert lib.cp_encode_jpeg(None, a.ctypes.data, 16, 16, 3, 95, 0, 0, None, 0,
                              _abi.ct.byref(size)) == _abi.CP_ERR_LIMIT
    assert size.value == len(cg.encode_jpeg(a))
    for bad in [(0, 16, 3, 95, 0), (16, 16, 2, 95, 0), (16, 16, 3, 101, 0), (16, 16, 3, 95, 2),
                (70000, 1, 3, 95, 0)]:
        w, h, c, q, ss = bad
        assert lib.cp_encode_jpeg(None, a.ctypes.data, w, h, c, q, ss, 0, None, 0,
                                  _abi.ct.byref(size)) == _abi.CP_ERR_ARG


# largest difference to the oracle per decoder route, in levels
TOLERANCE = {"engine": (3, 1), "software": (2, 1)}  # (RGB, gray)


def _header_error(tmp_path, data):
    p = tmp_path / "bad.jpg"
    p.write_bytes(data)
    with pytest.raises(cg.ChronoError) as e:
        cg.jpeg_info(p)
    assert e.value.status == _abi.CP_ERR_IO


def test_header_errors(tmp_path):
    """Missing, truncated and unsupported files are CP_ERR_IO before any decoding."""
    good = cg.encode_jpeg(gradient(16, 24))
    sof = good.index(b"\xff\xc0")
    _header_error(tmp_path, b"")
    _header_error(tmp_path, b"\x89PNG\r\n\x1a\n")
    _header_error(tmp_path, good[:sof + 6])                           # truncated frame header
    _header_error(tmp_path, good[:sof + 1] + b"\xc3" + good[sof + 2:])  # lossless process
    _header_error(tmp_path, good[:sof + 1] + b"\xc9" + good[sof + 2:])  # arithmetic coding
    _header_error(tmp_path, good[:sof + 4] + b"\x0c" + good[sof + 5:])  # 12-bit samples
    _header_error(tmp_path, good[:sof + 9] + b"\x04" + good[sof + 10:])  # 4 components
    with pytest.raises(cg.ChronoError) as e:
        cg.jpeg_info(tmp_path / "missing.jpg")
    assert e.value.status == _abi.CP_ERR_IO
    # progressive and extended-sequential headers are accepted (nvJPEG's software route)
    for m in (b"\xc1", b"\xc2"):
        p = tmp_path / "ok.jpg"
        p.write_bytes(good[:sof + 1] + m + good[sof + 2:])
        assert cg.jpeg_info(p) == (24, 16, 3)


def test_third_party_files_decode():
    """JPEG files from another encoder (scikit-learn's sample images, when installed) read
    through the oracle and cp_jpeg_info alike."""
    sk = pytest.importorskip("sklearn")
    d = os.path.join(os.path.dirname(sk.__file__), "datasets", "images")
    files = [os.path.join(d, f) for f in ("china.jpg", "flower.jpg")
             if os.path.exists(os.path.join(d, f))]
    if not files:
        pytest.skip("no sample images")
    for f in files:
        img = oracle.jpeg_decode(open(f, "rb").read())
        w, h, c = cg.jpeg_info(f)
        assert img.shape == (h, w, c) and c == 3 and 20 < img.mean() < 235


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="golden decodings not generated")
def test_oracle_matches_nvjpeg_golden():
    """The oracle's decoding of each golden file is within the stated tolerance of nvJPEG's
    (engines and software backend), and the encoder still writes the golden bytes."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_jpeg_golden", os.path.join(os.path.dirname(GOLDEN), "make_jpeg_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    g = np.load(GOLDEN)
    for name, h, w, c, q, ss, seed in mk.CASES:
        src = g[name + "/source"]
        assert np.array_equal(src, mk.image(h, w, c, seed))
        data = g[name + "/jpeg"].tobytes()
        assert cg.encode_jpeg(src, quality=q, subsampling=ss) == data, name
        ref = oracle.jpeg_decode(data).astype(int)
        for route in ("engine", "software"):
            nv = g[name + "/" + route].astype(int)
            assert nv.shape == ref.shape
            d = np.abs(nv - ref)
            tol = TOLERANCE[route][1 if c == 1 else 0]
            assert d.max() <= tol and d.mean() < 0.1, (name, route)
