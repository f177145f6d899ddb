"""Output encode (cp_save_png): the PNG files written must decode, with an independent
reader (chunk CRCs, Python's zlib, the PNG scanline filters restated here in Python), to
exactly the image that was saved, at every zlib level and for every block kind the
compressor picks (stored for noise, fixed or dynamic Huffman, long and overlapping
matches). CPU only: encoding needs no GPU."""
import os
import struct
import zlib

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi


def read_png(path):
    """Independent reader: returns (uint8 [h, w, c], filter types used)."""
    d = open(path, "rb").read()
    assert d[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, b"", None
    while pos < len(d):
        ln = struct.unpack(">I", d[pos:pos + 4])[0]
        typ, body = d[pos + 4:pos + 8], d[pos + 8:pos + 8 + ln]
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == struct.unpack(">I", d[pos + 8 + ln:pos + 12 + ln])[0]
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    w, h, depth, color, comp, filt, lace = hdr
    assert (depth, comp, filt, lace) == (8, 0, 0, 0)
    c = {0: 1, 2: 3, 6: 4}[color]
    raw = zlib.decompress(idat)
    stride = w * c
    assert len(raw) == h * (stride + 1)
    out = np.zeros((h, stride), np.int64)
    ftypes = []
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        f = raw[y * (stride + 1)]
        ftypes.append(f)
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int64)
        row = np.zeros(stride, np.int64)
        for i in range(stride):
            a = row[i - c] if i >= c else 0
            b = prev[i]
            cc = prev[i - c] if i >= c else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:
                pp = a + b - cc
                pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - cc)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else cc)
            row[i] = (line[i] + p) & 0xFF
        out[y] = row
        prev = row
    return out.astype(np.uint8).reshape(h, w, c), ftypes


def _images(c):
    rng = np.random.default_rng(c)
    yy, xx = np.mgrid[0:24, 0:40]
    smooth = np.stack([(xx * (k + 2) + yy * (5 - k)) % 256 for k in range(c)], -1)
    return {
        "noise": rng.integers(0, 256, size=(17, 23, c)),
        "smooth": smooth,
        "smooth+noise": (smooth + rng.integers(0, 4, size=smooth.shape)) % 256,
        "constant": np.full((9, 50, c), 77),
        "pixel": rng.integers(0, 256, size=(1, 1, c)),
        "column": rng.integers(0, 8, size=(30, 1, c)) * 30,
    }


@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_independent_reader_round_trip(tmp_path, c, level):
    for name, img in _images(c).items():
        img = img.astype(np.uint8)
        p = str(tmp_path / ("%s.png" % name))
        cg.save_png(p, img, level=level)
        got, ftypes = read_png(p)
        assert np.array_equal(got, img), name
        if level == 0:
            assert set(ftypes) == {0}
        assert np.array_equal(cg.load_png([p])[0], img), name


@pytest.mark.parametrize("level", [1, 6, 9])
def test_large_images_decode_and_compress(tmp_path, level):
    """1080p: a photo-like composite (many short matches), a flat one (runs of 258 at
    distance 1..4: overlapping copies), and noise (stored blocks chosen by cost)."""
    from chrono_photo_gb300 import example_data
    photo = example_data.hd_stack(seed=2, n=1)[0]
    flat = np.zeros_like(photo)
    flat[:, :, 0] = 200
    flat[500:600, 700:900] = (10, 20, 30)
    noise = np.random.default_rng(1).integers(0, 256, size=photo.shape, dtype=np.uint8)
    for name, img in (("photo", photo), ("flat", flat), ("noise", noise)):
        p = str(tmp_path / ("%s.png" % name))
        cg.save_png(p, img, level=level)
        assert np.array_equal(cg.load_png([p])[0], img), name
        chunks = open(p, "rb").read()
        # the zlib stream itself must be valid for an independent inflater
        idat = b"".join(chunks[i + 8:i + 8 + struct.unpack(">I", chunks[i:i + 4])[0]]
                        for i in _chunk_offsets(chunks) if chunks[i + 4:i + 8] == b"IDAT")
        assert len(zlib.decompress(idat)) == img.shape[0] * (img.shape[1] * 3 + 1)
        size = os.path.getsize(p)
        if name == "flat":
            assert size < img.nbytes / 500
        if name == "noise":
            assert size < img.nbytes * 1.01


def _chunk_offsets(d):
    pos = 8
    while pos < len(d):
        yield pos
        pos += 12 + struct.unpack(">I", d[pos:pos + 4])[0]


def test_creates_missing_parent_directory(tmp_path):
    img = np.full((4, 5, 3), 9, np.uint8)
    p = tmp_path / "new_dir" / "out.png"
    cg.save_png(str(p), img)
    assert np.array_equal(read_png(str(p))[0], img)
    with pytest.raises(cg.ChronoError) as e:  # like the reference: one level only
        cg.save_png(str(tmp_path / "a" / "b" / "out.png"), img)
    assert e.value.status == _abi.CP_ERR_IO


def test_invalid_arguments(tmp_path):
    with pytest.raises(cg.ChronoError) as e:
        cg.save_png(str(tmp_path / "x.png"), np.zeros((2, 2, 2), np.uint8))
    assert e.value.status == _abi.CP_ERR_ARG
    with pytest.raises(cg.ChronoError) as e:
        cg.save_png(str(tmp_path / "x.png"), np.zeros((2, 2, 3), np.uint8), level=10)
    assert e.value.status == _abi.CP_ERR_ARG


def test_all_block_kinds_are_exercised(tmp_path):
    """Across the small images the compressor picks stored (noise), fixed-Huffman (tiny or
    flat images) and dynamic-Huffman blocks: the round-trip tests above cover each kind."""
    kinds = set()
    for c in (1, 3, 4):
        for name, img in _images(c).items():
            p = str(tmp_path / "k.png")
            cg.save_png(p, img.astype(np.uint8), level=6)
            d = open(p, "rb").read()
            idat = b"".join(d[i + 8:i + 8 + struct.unpack(">I", d[i:i + 4])[0]]
                            for i in _chunk_offsets(d) if d[i + 4:i + 8] == b"IDAT")
            kinds.add((idat[2] >> 1) & 3)  # BTYPE of the first block
    assert kinds == {0, 1, 2}


def test_file_independent_of_thread_count(tmp_path):
    """Segments have a fixed size, so the bytes written do not depend on the threads used;
    a 1.3 MB image spans several segments (each primed with the 32 KB before it)."""
    from chrono_photo_gb300 import example_data
    img = example_data.stack(1, 640, 700, sigma=3, n_disks=2, rmin=20, rmax=40, seed=3)[0]
    files = []
    for t in (1, 3, 0):
        p = str(tmp_path / ("t%d.png" % t))
        cg.save_png(p, img, level=6, threads=t)
        files.append(open(p, "rb").read())
    assert files[0] == files[1] == files[2]
    assert np.array_equal(cg.load_png([str(tmp_path / "t1.png")])[0], img)


def test_directory_as_output_path(tmp_path):
    with pytest.raises(cg.ChronoError) as e:
        cg.save_png(str(tmp_path), np.zeros((2, 2, 3), np.uint8))
    assert e.value.status == _abi.CP_ERR_IO
