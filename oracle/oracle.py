"""ctypes binding of the CPU oracle (oracle/chrono_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the parity checker of the test suite and the smoke check, and the
timed CPU baseline of bench.py. The product library never imports it, and it imports nothing
of the product: the option and stack structs below are its own ctypes copies of the plain C
layouts that include/chrono_gpu.h declares (tests/test_abi.py checks that they match), and
`params()` builds the parsed options in Python, so a process that only runs the oracle maps
liboracle.so and no other library of this repository.
"""
import ctypes as ct
import os
import subprocess

import numpy as np

MODE = {"outlier": 0, "darker": 1, "lighter": 2}
OUTLIER = {"first": 0, "last": 1, "extreme": 2, "average": 3, "forward": 4, "backward": 5}
BACKGROUND = {"first": 0, "random": 1, "average": 2, "median": 3}


class Fade(ct.Structure):
    """cp_fade."""
    _fields_ = [("enabled", ct.c_int32), ("repeat", ct.c_int32), ("absolute", ct.c_int32),
                ("n_points", ct.c_int32), ("frames", ct.POINTER(ct.c_int32)),
                ("values", ct.POINTER(ct.c_float))]


class Params(ct.Structure):
    """cp_params: the parsed CLI options of one composite."""
    _fields_ = [("mode", ct.c_int32), ("thr_abs", ct.c_int32), ("thr_min", ct.c_float),
                ("thr_max", ct.c_float), ("outlier", ct.c_int32), ("background", ct.c_int32),
                ("weights", ct.c_float * 4), ("fade", Fade),
                ("sample", ct.POINTER(ct.c_int32)), ("n_sample", ct.c_int32),
                ("rng_seed", ct.c_uint64)]


class Stack(ct.Structure):
    """cp_stack."""
    _fields_ = [("n", ct.c_int32), ("width", ct.c_int32), ("height", ct.c_int32),
                ("channels", ct.c_int32), ("frames", ct.POINTER(ct.c_void_p)),
                ("base", ct.c_void_p), ("frame_stride", ct.c_int64),
                ("crop", ct.POINTER(ct.c_int32)), ("src_width", ct.c_int32),
                ("src_height", ct.c_int32), ("frame_offset", ct.c_int32)]


class Debug(ct.Structure):
    """cp_debug."""
    _fields_ = [("median", ct.c_void_p), ("q1", ct.c_void_p), ("q3", ct.c_void_p),
                ("outlier_bits", ct.c_void_p), ("chosen", ct.c_void_p),
                ("background", ct.c_void_p), ("n_outliers", ct.c_void_p)]


def params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme", background="random",
           weights=(1.0, 1.0, 1.0, 1.0), fade=None, sample=None, seed=0x5EED):
    """The parsed options of the reference's CLI as a cp_params, built in Python: defaults of
    src/cli.rs:192-216 (outlier, abs/0.05/0.2, background random, extreme, weights 1 1 1 1,
    no fade); `threshold` is "(abs|rel)/min[/max]" with max defaulting to min
    (src/options.rs:270-276); `fade` is "(clamp|repeat)/(abs|rel)/f,v/..." (src/options.rs:
    141-187). The buffers the struct points into travel on it as `_keep`."""
    p = Params()
    keep = []
    parts = threshold.split("/")
    if parts[0] not in ("abs", "absolute", "rel", "relative") or len(parts) < 2:
        raise ValueError("threshold must be (abs|rel)/min[/max]: %r" % threshold)
    p.mode = MODE[mode]
    p.thr_abs = 1 if parts[0].startswith("abs") else 0
    p.thr_min = float(parts[1])
    p.thr_max = float(parts[2]) if len(parts) > 2 else float(parts[1])
    p.outlier = OUTLIER[outlier]
    p.background = BACKGROUND[background]
    w = list(weights) + [1.0] * (4 - len(weights))
    for i in range(4):
        p.weights[i] = float(w[i])
    p.fade.absolute = 1  # FadeMode default of an absent --fade (unused while disabled)
    if fade:
        fp = fade.split("/")
        if fp[0] not in ("clamp", "repeat") or fp[1] not in ("abs", "absolute", "rel", "relative"):
            raise ValueError("fade must be (clamp|repeat)/(abs|rel)/f,v/...: %r" % fade)
        pts = [(int(a), float(b)) for a, b in (q.split(",") for q in fp[2:])]
        fr = (ct.c_int32 * len(pts))(*[a for a, _ in pts])
        va = (ct.c_float * len(pts))(*[b for _, b in pts])
        keep += [fr, va]
        p.fade.enabled = 1
        p.fade.repeat = 1 if fp[0] == "repeat" else 0
        p.fade.absolute = 1 if fp[1].startswith("abs") else 0
        p.fade.n_points = len(pts)
        p.fade.frames = ct.cast(fr, ct.POINTER(ct.c_int32))
        p.fade.values = ct.cast(va, ct.POINTER(ct.c_float))
    if sample is not None and len(sample) > 0:
        arr = (ct.c_int32 * len(sample))(*[int(s) for s in sample])
        keep.append(arr)
        p.sample = ct.cast(arr, ct.POINTER(ct.c_int32))
        p.n_sample = len(sample)
    p.rng_seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    p._keep = keep
    return p


def _addr(s):
    """Address of a ctypes struct: the oracle takes the C layouts by pointer, whichever
    Python class (this module's or the product binding's) describes them."""
    return None if s is None else ct.addressof(s)


HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRCS = [os.path.join(HERE, "chrono_oracle.cpp"), os.path.join(HERE, "jpeg_oracle.cpp")]

_lib = None


def build():
    """Compile liboracle.so with -ffp-contract=off (f32 ops rounded one by one, like rustc)."""
    hdr = os.path.join(HERE, "..", "include", "chrono_gpu.h")
    if (not os.path.exists(LIB)
            or any(os.path.getmtime(LIB) < os.path.getmtime(f) for f in SRCS + [hdr])):
        cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fPIC", "-pthread",
               "-ffp-contract=off", "-fno-fast-math", "-shared", "-o", LIB + ".tmp"] + SRCS
        subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        l = ct.CDLL(LIB)
        P = ct.c_void_p
        l.or_quartiles.argtypes = [P, ct.c_int32, ct.POINTER(ct.c_float), ct.POINTER(ct.c_float),
                                   ct.POINTER(ct.c_float)]
        l.or_jpeg_info.argtypes = [P, ct.c_size_t, ct.POINTER(ct.c_int32),
                                   ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int32)]
        l.or_jpeg_decode.argtypes = [P, ct.c_size_t, P, ct.c_size_t]
        l.or_median.argtypes = [P, ct.c_int32]
        l.or_median.restype = ct.c_float
        l.or_blend_value.argtypes = [ct.c_int32, ct.c_float, ct.c_float, ct.c_float]
        l.or_blend_value.restype = ct.c_float
        l.or_threshold.argtypes = [ct.c_int32, ct.c_float, ct.c_float, ct.POINTER(ct.c_float)]
        l.or_blend_into_u8.argtypes = [P, P, ct.c_int32, ct.c_float]
        l.or_gen_range.argtypes = [ct.c_uint64, ct.c_uint64, ct.c_uint32]
        l.or_gen_range.restype = ct.c_uint32
        l.or_fade_lut.argtypes = [P, ct.c_int32, ct.c_int32, ct.POINTER(ct.c_float)]
        l.or_composite.argtypes = [P, P, P, P, P, ct.POINTER(ct.c_uint64), ct.c_int32]
        l.or_shake_analyze.argtypes = [ct.POINTER(P), ct.c_int32, ct.c_int32, ct.c_int32,
                                       ct.c_int32, P, ct.c_int32, ct.c_int32, ct.c_int32, P, P,
                                       ct.c_int32]
        l.or_crop_create.argtypes = [P, ct.c_int32, ct.c_int32, ct.c_int32, P, P]
        l.or_video_windows.argtypes = [ct.c_int32] * 11 + [ct.POINTER(ct.c_int32),
                                                           ct.POINTER(ct.c_int64), P, P, P, P]
        _lib = l
    return _lib


def fade_lut(fade, n, frame_offset=0):
    """fade(i, n, frame_offset) of every sample from a cp_fade struct."""
    o = (ct.c_float * n)()
    if lib().or_fade_lut(_addr(fade), n, frame_offset, o) != 0:
        raise ValueError("invalid fade")
    return np.frombuffer(o, np.float32).copy()


def quartiles(sorted_values):
    a = np.ascontiguousarray(sorted_values, dtype=np.uint8)
    q1, md, q3 = ct.c_float(), ct.c_float(), ct.c_float()
    rc = lib().or_quartiles(a.ctypes.data, len(a), ct.byref(q1), ct.byref(md), ct.byref(q3))
    if rc != 0:
        raise ValueError("quartiles need at least 3 values")
    return q1.value, md.value, q3.value


def composite(frames, params, frame_offset=0, crop=None, out_size=None, threads=1, debug=False):
    """OutlierProcessor / SimpleProcessor restated on the CPU. frames: uint8 [n, h, w, c].
    Returns (composite, blend mask, warnings[, debug dict])."""
    a = np.ascontiguousarray(frames, dtype=np.uint8)
    n, h, w, c = a.shape
    st = Stack()
    st.n, st.channels = n, c
    st.base = a.ctypes.data
    st.frame_stride = h * w * c
    st.frame_offset = frame_offset
    keep = []
    if crop is not None:
        origins = np.ascontiguousarray(np.asarray(crop, dtype=np.int32).reshape(-1))
        keep.append(origins)
        st.crop = origins.ctypes.data_as(ct.POINTER(ct.c_int32))
        st.src_width, st.src_height = w, h
        w, h = out_size
    st.width, st.height = w, h
    out = np.empty((h, w, c), np.uint8)
    blend = np.empty((h, w, c), np.uint8)
    warn = ct.c_uint64()
    dbg = None
    arrays = None
    if debug:
        words = (n + 31) // 32
        arrays = {"median": np.zeros((h, w, c), np.float32), "q1": np.zeros((h, w, c), np.float32),
                  "q3": np.zeros((h, w, c), np.float32),
                  "outlier_bits": np.zeros((h, w, words), np.uint32),
                  "chosen": np.zeros((h, w), np.int32), "background": np.zeros((h, w), np.int32),
                  "n_outliers": np.zeros((h, w), np.int32)}
        dbg = Debug(*[arrays[k].ctypes.data for k in ("median", "q1", "q3", "outlier_bits",
                                                            "chosen", "background", "n_outliers")])
    rc = lib().or_composite(_addr(st), _addr(params), out.ctypes.data, blend.ctypes.data,
                            _addr(dbg), ct.byref(warn), threads)
    if rc != 0:
        raise ValueError("oracle rejected the stack (%d)" % rc)
    if debug:
        return out, blend, warn.value, arrays
    return out, blend, warn.value


def shake(frames, anchors, r, s, threads=1, diffs=False):
    """ShakeAnalyzer::analyze restated: (offsets [n, 2][, diffs [n-1, S, S]])."""
    a = np.ascontiguousarray(frames, dtype=np.uint8)
    n, h, w, c = a.shape
    ptrs = (ct.c_void_p * n)(*[a[i].ctypes.data for i in range(n)])
    anc = np.ascontiguousarray(np.asarray(anchors, dtype=np.int32).reshape(-1))
    offs = np.zeros((n, 2), np.int32)
    S = 2 * s + 1
    dd = np.zeros((max(n - 1, 0), S, S), np.int32)
    rc = lib().or_shake_analyze(ptrs, n, w, h, c, anc.ctypes.data, len(anc) // 2, r, s,
                                offs.ctypes.data, dd.ctypes.data, threads)
    if rc != 0:
        raise ValueError("oracle shake failed (%d)" % rc)
    return (offs, dd) if diffs else offs


def crop_create(offsets, width, height):
    offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32).reshape(-1))
    has = ct.c_int32()
    crops = np.zeros((len(offs) // 2, 4), np.int32)
    lib().or_crop_create(offs.ctypes.data, len(offs) // 2, width, height, ct.byref(has),
                         crops.ctypes.data)
    return crops if has.value else None


def video_windows(image_count, video_in, video_out=(None, None, 1)):
    (a, b, s), (c, d, t) = video_in, video_out
    nw, ni = ct.c_int32(), ct.c_int64()
    args = [image_count, int(a is not None), a or 0, int(b is not None), b or 0, s or 1,
            int(c is not None), c or 0, int(d is not None), d or 0, t or 1]
    lib().or_video_windows(*args, ct.byref(nw), ct.byref(ni), None, None, None, None)
    k = max(nw.value, 1)
    starts, lens, frames = np.zeros(k, np.int64), np.zeros(k, np.int32), np.zeros(k, np.int32)
    idx = np.zeros(max(ni.value, 1), np.int32)
    lib().or_video_windows(*args, ct.byref(nw), ct.byref(ni), starts.ctypes.data, lens.ctypes.data,
                           idx.ctypes.data, frames.ctypes.data)
    return [(int(frames[i]), [int(v) for v in idx[starts[i]:starts[i] + lens[i]]])
            for i in range(nw.value)]


def jpeg_decode(data):
    """A sequential (baseline or extended) JPEG file's bytes decoded by the exact-IDCT
    reference decoder (jpeg_oracle.cpp): uint8 [h, w, c], c = 1 or 3."""
    buf = np.frombuffer(bytes(data), np.uint8)
    w, h, c = ct.c_int32(), ct.c_int32(), ct.c_int32()
    l = lib()
    if l.or_jpeg_info(buf.ctypes.data, buf.size, ct.byref(w), ct.byref(h), ct.byref(c)) != 0:
        raise ValueError("not a sequential 8-bit JPEG the oracle reads")
    out = np.empty((h.value, w.value, c.value), np.uint8)
    if l.or_jpeg_decode(buf.ctypes.data, buf.size, out.ctypes.data, out.nbytes) != 0:
        raise ValueError("corrupt JPEG data")
    return out
