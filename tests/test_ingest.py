"""Frame ingest (cp_load_png / cp_png_info): PNG files written here by an independent encoder
(zlib + the five scanline filters of the PNG specification, chosen per row) must decode to
exactly the arrays they were written from; unsupported or damaged files fail with
CP_ERR_IO. CPU only: decoding needs no GPU."""
import struct
import zlib

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi

COLOR_TYPE = {1: 0, 3: 2, 4: 6}


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(
        ">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(img, rng):
    """Filtered scanlines (filter byte + bytes) with a random filter type per row."""
    h, w, c = img.shape
    rows = img.reshape(h, w * c).astype(np.int32)
    out = bytearray()
    prev = np.zeros(w * c, np.int32)
    for y in range(h):
        x = rows[y]
        a = np.concatenate([np.zeros(c, np.int32), x[:-c]])
        b = prev
        cc = np.concatenate([np.zeros(c, np.int32), prev[:-c]])
        ft = int(rng.integers(0, 5))
        pred = [np.zeros_like(x), a, b, (a + b) // 2, _paeth(a, b, cc)][ft]
        out.append(ft)
        out += ((x - pred) & 0xFF).astype(np.uint8).tobytes()
        prev = x
    return bytes(out)


def _deflate(raw, level, strategy):
    z = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    return z.compress(raw) + z.flush()


def write_png(path, img, seed=0, level=6, idat_parts=1, text=False, header=None,
              strategy=zlib.Z_DEFAULT_STRATEGY, filters=True, damage=None):
    """img: uint8 [h, w, c]. header: optional (depth, color, interlace) override.
    filters=False writes every row with filter type 0; damage(data) may alter the zlib
    stream before it is split into IDAT chunks (with valid chunk CRCs)."""
    h, w, c = img.shape
    depth, color, lace = header or (8, COLOR_TYPE[c], 0)
    if filters:
        raw = _filter_rows(img, np.random.default_rng(seed))
    else:
        raw = np.concatenate([np.zeros((h, 1), np.uint8), img.reshape(h, w * c)], 1).tobytes()
    data = _deflate(raw, level, strategy)
    if damage:
        data = damage(data)
    parts = np.array_split(np.frombuffer(data, np.uint8), idat_parts)
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0,
                                                              0, lace))
    if text:
        png += _chunk(b"tEXt", b"Comment\x00written by the ingest tests")
    if color == 3:
        png += _chunk(b"PLTE", bytes(range(48)))
    for part in parts:
        png += _chunk(b"IDAT", part.tobytes())
    png += _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)
    return path


@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (21, 37), (64, 200)])
def test_round_trip(tmp_path, c, shape):
    rng = np.random.default_rng(shape[0] * 10 + c)
    n = 5
    frames = rng.integers(0, 256, size=(n, shape[0], shape[1], c), dtype=np.uint8)
    paths = [write_png(str(tmp_path / ("f%d.png" % i)), frames[i], seed=i, level=i % 10)
             for i in range(n)]
    assert cg.png_info(paths[0]) == (shape[1], shape[0], c)
    for threads in (1, 3, 0):
        got = cg.load_png(paths, threads=threads)
        assert np.array_equal(got, frames)


def _photo_like(h, w, c, seed):
    """Smooth gradients with a little noise and repeated patches: compresses with many
    back-references, as camera frames do."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    base = np.stack([(x * (k + 1) + y * (3 - k)) // 4 for k in range(c)], -1)
    img = (base + rng.integers(0, 3, size=(h, w, c))) % 256
    k = min(8, h - h // 3)
    img[h // 3: h // 3 + k] = img[:k]
    return img.astype(np.uint8)


@pytest.mark.parametrize("strategy", [zlib.Z_DEFAULT_STRATEGY, zlib.Z_FILTERED,
                                      zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE, zlib.Z_FIXED],
                         ids=["default", "filtered", "huffman-only", "rle", "fixed"])
@pytest.mark.parametrize("level", [1, 6, 9])
def test_deflate_block_kinds(tmp_path, strategy, level):
    """Dynamic and fixed Huffman blocks, short and long matches, overlapping runs."""
    frames = np.stack([_photo_like(48, 300, 3, s) for s in range(3)])
    paths = [write_png(str(tmp_path / ("d%d.png" % i)), frames[i], seed=i, level=level,
                       strategy=strategy, filters=i != 1) for i in range(3)]
    assert np.array_equal(cg.load_png(paths, threads=2), frames)


def test_long_distance_and_stored_blocks(tmp_path):
    """Rows of 24000 bytes repeated: matches reach back ~24 KB (the distance codes with the
    most extra bits); level 0 gives stored blocks of up to 64 KB, several per image."""
    row = np.random.default_rng(9).integers(0, 256, size=(1, 8000, 3), dtype=np.uint8)
    img = np.repeat(row, 6, 0)
    img[3, 100:200] ^= 0x5A
    for level in (0, 9):
        p = write_png(str(tmp_path / ("l%d.png" % level)), img, level=level, filters=False)
        assert np.array_equal(cg.load_png([p])[0], img)


def test_split_data_and_ancillary_chunks(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, size=(40, 33, 3), dtype=np.uint8)
    p = write_png(str(tmp_path / "a.png"), img, idat_parts=7, text=True)
    assert np.array_equal(cg.load_png([p])[0], img)


def test_into_preallocated_stack(tmp_path):
    rng = np.random.default_rng(4)
    frames = rng.integers(0, 256, size=(3, 9, 11, 4), dtype=np.uint8)
    paths = [write_png(str(tmp_path / ("g%d.png" % i)), frames[i]) for i in range(3)]
    out = np.zeros_like(frames)
    assert cg.load_png(paths, out=out) is out
    assert np.array_equal(out, frames)


def _expect_io(paths):
    with pytest.raises(cg.ChronoError) as e:
        cg.load_png(paths)
    assert e.value.status == _abi.CP_ERR_IO


@pytest.mark.parametrize("header", [(8, 2, 1), (16, 2, 0), (8, 3, 0), (8, 4, 0)],
                         ids=["interlaced", "16-bit", "palette", "gray-alpha"])
def test_unsupported_formats(tmp_path, header):
    good = write_png(str(tmp_path / "good.png"), np.zeros((4, 4, 3), np.uint8))
    bad = write_png(str(tmp_path / "bad.png"), np.zeros((4, 4, 3), np.uint8), header=header)
    with pytest.raises(cg.ChronoError) as e:
        cg.png_info(bad)
    assert e.value.status == _abi.CP_ERR_IO
    _expect_io([good, bad])


def test_damaged_and_mismatched_files(tmp_path):
    img = np.random.default_rng(5).integers(0, 256, size=(16, 16, 3), dtype=np.uint8)
    good = write_png(str(tmp_path / "good.png"), img)
    raw = open(good, "rb").read()
    trunc = tmp_path / "trunc.png"
    trunc.write_bytes(raw[:len(raw) // 2])
    crc = bytearray(raw)
    crc[40] ^= 0xFF  # inside the IDAT payload: its CRC no longer matches
    badcrc = tmp_path / "crc.png"
    badcrc.write_bytes(bytes(crc))
    other = write_png(str(tmp_path / "other.png"), img[:8])
    for p in (str(trunc), str(badcrc), str(tmp_path / "missing.png"), other):
        _expect_io([good, p])


def _flip(i, mask=0x01):
    def damage(d):
        d = bytearray(d)
        d[i] ^= mask
        return bytes(d)
    return damage


@pytest.mark.parametrize("damage", [
    _flip(-1),                                     # Adler-32 of the data
    _flip(0, 0x07),                                # zlib header: compression method
    _flip(1, 0x20),                                # zlib header: preset dictionary flag
    lambda d: d[:-9],                              # DEFLATE stream cut short
    lambda d: d[:2] + bytes([0x07]) + d[3:],       # final block of reserved type 3
], ids=["adler", "method", "dictionary", "cut", "block-type"])
def test_damaged_zlib_stream(tmp_path, damage):
    """Chunk CRCs are valid here: the zlib layer itself must catch each defect."""
    img = _photo_like(24, 50, 3, 1)
    good = write_png(str(tmp_path / "good.png"), img, level=9)
    bad = write_png(str(tmp_path / "bad.png"), img, level=9, damage=damage)
    _expect_io([good, bad])


def test_image_data_longer_than_the_image(tmp_path):
    img = _photo_like(8, 10, 3, 2)
    bigger = _photo_like(9, 10, 3, 2)
    raw = np.concatenate([np.zeros((9, 1), np.uint8), bigger.reshape(9, 30)], 1).tobytes()
    p = write_png(str(tmp_path / "x.png"), img, damage=lambda d: zlib.compress(raw))
    _expect_io([p])
    with pytest.raises(cg.ChronoError):
        cg.load_png([str(tmp_path / "missing.png")])


def test_damaged_streams_fail_cleanly(tmp_path):
    """Random damage to the zlib data (bytes flipped, cut, inserted; chunk CRCs kept valid so
    that the DEFLATE decoder itself meets it): every file either decodes or fails with
    CP_ERR_IO, never anything else."""
    rng = np.random.default_rng(11)
    p = str(tmp_path / "f.png")
    outcomes = {0: 0, _abi.CP_ERR_IO: 0}
    for it in range(300):
        h, w, c = int(rng.integers(1, 30)), int(rng.integers(1, 40)), int(rng.choice([1, 3, 4]))
        img = (_photo_like(h, w, c, it) if it % 2 else
               rng.integers(0, 256, size=(h, w, c), dtype=np.uint8))

        def damage(data):
            b = bytearray(data)
            kind = int(rng.integers(0, 3))
            if kind == 0:
                for _ in range(int(rng.integers(1, 4))):
                    b[int(rng.integers(0, len(b)))] ^= int(rng.integers(1, 256))
            elif kind == 1:
                b = b[:int(rng.integers(0, len(b)))]
            else:
                i = int(rng.integers(0, len(b)))
                b[i:i] = rng.integers(0, 256, size=int(rng.integers(1, 20)), dtype=np.uint8).tobytes()
            return bytes(b)
        write_png(p, img, seed=it, level=int(rng.integers(0, 10)),
                  strategy=int(rng.choice([0, 1, 2, 3, 4])), damage=damage)
        try:
            cg.load_png([p])
            outcomes[0] += 1
        except cg.ChronoError as e:
            assert e.status == _abi.CP_ERR_IO, e
            outcomes[_abi.CP_ERR_IO] += 1
    assert outcomes[_abi.CP_ERR_IO] > 250


def test_directory_is_not_a_frame(tmp_path):
    """A directory given as a frame path is an I/O error, not a crash."""
    d = tmp_path / "subdir"
    d.mkdir()
    with pytest.raises(cg.ChronoError) as e:
        cg.png_info(str(d))
    assert e.value.status == _abi.CP_ERR_IO
    good = write_png(str(tmp_path / "g.png"), np.zeros((2, 2, 3), np.uint8))
    _expect_io([good, str(d)])
