"""ctypes binding of the CPU oracle (oracle/chrono_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the parity checker of the test suite and the smoke check, and the
timed CPU baseline of bench.py. The product library never imports it.
"""
import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "chrono_oracle.cpp")

_lib = None


def build():
    """Compile liboracle.so with -ffp-contract=off (f32 ops rounded one by one, like rustc)."""
    hdr = os.path.join(HERE, "..", "include", "chrono_gpu.h")
    if (not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC)
            or os.path.getmtime(LIB) < os.path.getmtime(hdr)):
        cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fPIC", "-pthread",
               "-ffp-contract=off", "-fno-fast-math", "-shared", "-o", LIB + ".tmp", SRC]
        subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        from chrono_photo_gb300 import _abi
        l = ct.CDLL(LIB)
        P = ct.c_void_p
        l.or_quartiles.argtypes = [P, ct.c_int32, ct.POINTER(ct.c_float), ct.POINTER(ct.c_float),
                                   ct.POINTER(ct.c_float)]
        l.or_median.argtypes = [P, ct.c_int32]
        l.or_median.restype = ct.c_float
        l.or_blend_value.argtypes = [ct.c_int32, ct.c_float, ct.c_float, ct.c_float]
        l.or_blend_value.restype = ct.c_float
        l.or_threshold.argtypes = [ct.c_int32, ct.c_float, ct.c_float, ct.POINTER(ct.c_float)]
        l.or_blend_into_u8.argtypes = [P, P, ct.c_int32, ct.c_float]
        l.or_gen_range.argtypes = [ct.c_uint64, ct.c_uint64, ct.c_uint32]
        l.or_gen_range.restype = ct.c_uint32
        l.or_fade_lut.argtypes = [ct.POINTER(_abi.Fade), ct.c_int32, ct.c_int32, ct.POINTER(ct.c_float)]
        l.or_composite.argtypes = [ct.POINTER(_abi.Stack), ct.POINTER(_abi.Params), P, P,
                                   ct.POINTER(_abi.Debug), ct.POINTER(ct.c_uint64), ct.c_int32]
        l.or_shake_analyze.argtypes = [ct.POINTER(P), ct.c_int32, ct.c_int32, ct.c_int32,
                                       ct.c_int32, P, ct.c_int32, ct.c_int32, ct.c_int32, P, P,
                                       ct.c_int32]
        l.or_crop_create.argtypes = [P, ct.c_int32, ct.c_int32, ct.c_int32, P, P]
        l.or_video_windows.argtypes = [ct.c_int32] * 11 + [ct.POINTER(ct.c_int32),
                                                           ct.POINTER(ct.c_int64), P, P, P, P]
        _lib = l
    return _lib


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
    from chrono_photo_gb300 import _abi
    a = np.ascontiguousarray(frames, dtype=np.uint8)
    n, h, w, c = a.shape
    st = _abi.Stack()
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
        dbg = _abi.Debug(*[arrays[k].ctypes.data for k in ("median", "q1", "q3", "outlier_bits",
                                                            "chosen", "background", "n_outliers")])
    rc = lib().or_composite(ct.byref(st), ct.byref(params), out.ctypes.data, blend.ctypes.data,
                            ct.byref(dbg) if dbg is not None else None, ct.byref(warn), threads)
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
