"""Python host API over libchrono_gpu.so, mirroring the reference's processor interface.

    chrono-photo (Rust)                          this module
    Threshold::abs/rel (src/options.rs:189-244)  Threshold
    Fade (src/options.rs:60-139)                 Fade
    OutlierProcessor::new/process (chrono.rs)    OutlierProcessor(...).process(frames)
    SimpleProcessor::new/process (simple.rs)     SimpleProcessor(...).process(frames)
    ShakeAnalyzer::analyze (shake.rs:190-313)    ShakeAnalyzer().analyze(frames, ...)
    Crop::create (shake.rs:136-176)              Crop.create(offsets, width, height)

Frames are numpy uint8 arrays [n, height, width, channels] (or a list of [h, w, c] arrays):
the decoded images the reference reads through `image::open`; the processors also take a
list of PNG or JPEG file paths, as the reference's take files (PNG decoded by cp_load_png on
host threads, JPEG by nvJPEG on the GPU straight into device frames). Every composite runs on
the GPU; there is no CPU path.
"""
import ctypes as ct
import os

import numpy as np

from . import _abi
from ._abi import ChronoError, lib


def _check(ctx, rc, what=""):
    if rc != _abi.CP_OK:
        msg = what
        if ctx is not None:
            buf = ct.create_string_buffer(512)
            lib().cp_ctx_last_error(ctx, buf, 512)
            if buf.value:
                msg = (what + ": " if what else "") + buf.value.decode()
        raise ChronoError(rc, msg)


class Threshold:
    """`(abs|rel)/min[/max]`; max defaults to min as the reference's parser does."""

    def __init__(self, absolute=True, min=0.05, max=None):
        self.absolute = bool(absolute)
        self.min = float(min)
        self.max = float(min if max is None else max)

    @classmethod
    def abs(cls, mn, mx=None):
        return cls(True, mn, mx)

    @classmethod
    def rel(cls, mn, mx=None):
        return cls(False, mn, mx)

    @classmethod
    def parse(cls, s):
        parts = s.split("/")
        if parts[0] not in ("abs", "absolute", "rel", "relative") or len(parts) < 2:
            raise ValueError("threshold must be (abs|rel)/min[/max]: %r" % s)
        return cls(parts[0].startswith("abs"), float(parts[1]),
                   float(parts[2]) if len(parts) > 2 else None)


class Fade:
    """`(clamp|repeat)/(abs|rel)/f,v/...`; Fade.none() is the default (all 1)."""

    def __init__(self, repeat=False, absolute=True, points=()):
        self.repeat = bool(repeat)
        self.absolute = bool(absolute)
        self.points = [(int(f), float(v)) for f, v in points]
        self.enabled = len(self.points) > 0

    @classmethod
    def none(cls):
        return cls()

    @classmethod
    def parse(cls, s):
        parts = s.split("/")
        if parts[0] not in ("clamp", "repeat") or parts[1] not in ("abs", "absolute", "rel", "relative"):
            raise ValueError("fade must be (clamp|repeat)/(abs|rel)/f,v/...: %r" % s)
        pts = []
        for p in parts[2:]:
            f, v = p.split(",")
            pts.append((int(f), float(v)))
        return cls(parts[0] == "repeat", parts[1].startswith("abs"), pts)

    def to_c(self, keep):
        f = _abi.Fade()
        f.enabled = 1 if self.enabled else 0
        f.repeat = 1 if self.repeat else 0
        f.absolute = 1 if self.absolute else 0
        f.n_points = len(self.points)
        if self.enabled:
            fr = (ct.c_int32 * len(self.points))(*[p[0] for p in self.points])
            va = (ct.c_float * len(self.points))(*[p[1] for p in self.points])
            keep += [fr, va]
            f.frames = ct.cast(fr, ct.POINTER(ct.c_int32))
            f.values = ct.cast(va, ct.POINTER(ct.c_float))
        return f

    def lut(self, n, frame_offset=0):
        """fade(i, n, frame_offset) for every sample i (src/chrono.rs:496-502)."""
        keep = []
        f = self.to_c(keep)
        out = (ct.c_float * n)()
        _check(None, lib().cp_fade_lut(ct.byref(f), n, frame_offset, out), "fade")
        return np.frombuffer(out, dtype=np.float32).copy()


def make_params(mode="outlier", threshold=None, outlier="extreme", background="random",
                weights=(1.0, 1.0, 1.0, 1.0), fade=None, sample=None, seed=0x5EED, keep=None):
    """cp_params from CLI-style values (defaults of src/cli.rs:192-216)."""
    keep = keep if keep is not None else []
    p = _abi.Params()
    lib().cp_params_default(ct.byref(p))
    threshold = threshold or Threshold.abs(0.05, 0.2)
    if isinstance(threshold, str):
        threshold = Threshold.parse(threshold)
    p.mode = _abi.MODE[mode]
    p.thr_abs = 1 if threshold.absolute else 0
    p.thr_min = threshold.min
    p.thr_max = threshold.max
    p.outlier = _abi.OUTLIER[outlier]
    p.background = _abi.BACKGROUND[background]
    w = list(weights) + [1.0] * (4 - len(weights))
    for i in range(4):
        p.weights[i] = float(w[i])
    if isinstance(fade, str):
        fade = Fade.parse(fade)
    p.fade = (fade or Fade.none()).to_c(keep)
    if sample is not None and len(sample) > 0:
        arr = (ct.c_int32 * len(sample))(*[int(s) for s in sample])
        keep.append(arr)
        p.sample = ct.cast(arr, ct.POINTER(ct.c_int32))
        p.n_sample = len(sample)
    p.rng_seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return p


def _is_paths(frames):
    return isinstance(frames, (list, tuple)) and len(frames) > 0 and \
        all(isinstance(f, (str, os.PathLike)) for f in frames)


_JPEG_EXT = (".jpg", ".jpeg", ".jpe", ".jfif")


def _is_jpeg(path):
    return str(path).lower().endswith(_JPEG_EXT)


def _as_stack(frames):
    """uint8 [n, h, w, c] from an array, a sequence of images, or a sequence of PNG or JPEG
    file paths (PNG decoded by cp_load_png on all host threads, JPEG by cp_load_jpeg on the
    GPU, as the reference's processors take their frames as files)."""
    if _is_paths(frames):
        if all(_is_jpeg(f) for f in frames):
            return load_jpeg(frames)
        if any(_is_jpeg(f) for f in frames):
            raise ValueError("a stack of files is all JPEG or all PNG")
        return load_png(frames)
    if isinstance(frames, np.ndarray):
        a = np.ascontiguousarray(frames, dtype=np.uint8)
        if a.ndim == 3:
            a = a[..., None]
        return a
    return np.ascontiguousarray(np.stack([np.asarray(f, dtype=np.uint8) for f in frames]))


def _select(frames, image_indices):
    """The frames at image_indices (all when None) and their frame offset
    (src/chrono.rs:103). File paths stay paths (selected before decoding, and decoded by
    Context.composite: JPEG straight into device memory); anything else becomes a stack."""
    if image_indices is None:
        return (list(frames) if _is_paths(frames) else _as_stack(frames)), 0
    idx = [int(i) for i in image_indices]
    if _is_paths(frames):
        return [frames[i] for i in idx], idx[0]
    return np.ascontiguousarray(_as_stack(frames)[idx]), idx[0]


class Context:
    """One device context (cp_ctx): streams, device memory accounting, staging buffers."""

    def __init__(self, device=0, hbm_budget=0):
        h = ct.c_void_p()
        rc = lib().cp_ctx_create(device, hbm_budget, ct.byref(h))
        _check(None, rc, "cp_ctx_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib().cp_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc, what=""):
        _check(self.handle, rc, what)

    # ---- device memory ------------------------------------------------------------------
    def alloc(self, nbytes):
        p = ct.c_void_p()
        self.check(lib().cp_dev_alloc(self.handle, nbytes, ct.byref(p)), "cp_dev_alloc")
        return p.value

    def free(self, ptr):
        self.check(lib().cp_dev_free(self.handle, ptr), "cp_dev_free")

    def upload(self, arr, ptr=None):
        arr = np.ascontiguousarray(arr)
        # 16 spare bytes: the kernels' 16-byte row copies may read past a frame's last pixel
        ptr = ptr or self.alloc(arr.nbytes + 16)
        self.check(lib().cp_memcpy_h2d(self.handle, ptr, arr.ctypes.data, arr.nbytes, None), "h2d")
        return ptr

    def download(self, ptr, shape, dtype=np.uint8):
        out = np.empty(shape, dtype=dtype)
        self.check(lib().cp_memcpy_d2h(self.handle, out.ctypes.data, ptr, out.nbytes, None), "d2h")
        return out

    def synchronize(self):
        self.check(lib().cp_ctx_synchronize(self.handle), "synchronize")

    # ---- compositing --------------------------------------------------------------------
    def composite(self, frames, params=None, blend=True, debug=False, crop=None,
                  src_size=None, frame_offset=0, **kw):
        """Host-memory composite of one stack (cp_composite). Returns
        (composite, blend_mask or None, warnings[, debug dict])."""
        keep = []
        p = params if params is not None else make_params(keep=keep, **kw)
        if (_is_paths(frames) and all(_is_jpeg(f) for f in frames) and not debug
                and crop is None):
            return self._composite_jpeg(frames, p, blend, frame_offset)
        a = _as_stack(frames)
        n, h, w, c = a.shape
        st = _abi.Stack()
        st.n = n
        st.channels = c
        st.base = a.ctypes.data
        st.frame_stride = h * w * c
        st.frame_offset = frame_offset
        if crop is not None:
            cw, chh = src_size if src_size else (None, None)
            ow, oh = crop[1]
            origins = np.ascontiguousarray(np.asarray(crop[0], dtype=np.int32).reshape(-1))
            keep.append(origins)
            st.crop = origins.ctypes.data_as(ct.POINTER(ct.c_int32))
            st.src_width, st.src_height = w, h
            st.width, st.height = ow, oh
            h, w = oh, ow
        else:
            st.width, st.height = w, h
        out = np.empty((h, w, c), dtype=np.uint8)
        bl = np.empty((h, w, c), dtype=np.uint8) if blend and p.mode == 0 else None
        warn = ct.c_uint64(0)
        dbg_arrays = None
        dbg = None
        if debug:
            words = (n + 31) // 32
            dbg_arrays = {
                "median": np.zeros((h, w, c), np.float32),
                "q1": np.zeros((h, w, c), np.float32),
                "q3": np.zeros((h, w, c), np.float32),
                "outlier_bits": np.zeros((h, w, words), np.uint32),
                "chosen": np.zeros((h, w), np.int32),
                "background": np.zeros((h, w), np.int32),
                "n_outliers": np.zeros((h, w), np.int32),
            }
            dbg = _abi.Debug(*[dbg_arrays[k].ctypes.data for k in
                               ("median", "q1", "q3", "outlier_bits", "chosen", "background",
                                "n_outliers")])
        rc = lib().cp_composite(self.handle, ct.byref(st), ct.byref(p), out.ctypes.data,
                                bl.ctypes.data if bl is not None else None,
                                ct.byref(dbg) if dbg is not None else None, ct.byref(warn))
        self.check(rc, "cp_composite")
        if debug:
            return out, bl, warn.value, dbg_arrays
        return out, bl, warn.value

    def load_jpeg_device(self, paths, threads=0):
        """Decodes JPEG files on the GPU (cp_load_jpeg_device) into one new device buffer:
        returns (pointer, frame_stride, (n, h, w, c)); frames start on 16-byte boundaries
        with 16 spare bytes after the last, as the compositing kernels read them. Free the
        buffer with free()."""
        paths = [str(f) for f in paths]
        if not paths:
            raise ValueError("no frames")
        w, h, c = jpeg_info(paths[0])
        fb = w * h * c
        stride = (fb + 15) // 16 * 16
        dev = self.alloc(len(paths) * stride + 16)
        try:
            arr = (ct.c_char_p * len(paths))(*[f.encode() for f in paths])
            self.check(lib().cp_load_jpeg_device(self.handle, arr, len(paths), int(threads), dev,
                                                 stride, w, h, c), "cp_load_jpeg_device")
        except Exception:
            self.free(dev)
            raise
        return dev, stride, (len(paths), h, w, c)

    def _composite_jpeg(self, paths, p, blend, frame_offset):
        """JPEG files -> composite with the frames decoded into device memory (only the
        compressed bytes cross the host link), then cp_composite_device and the results
        copied back."""
        dev, stride, (n, h, w, c) = self.load_jpeg_device(paths)
        ptrs = [dev]
        try:
            fb = h * w * c
            out_d = self.alloc(fb)
            ptrs.append(out_d)
            bl_d = None
            if blend and p.mode == 0:
                bl_d = self.alloc(fb)
                ptrs.append(bl_d)
            warn_d = self.upload(np.zeros(1, np.uint64))
            ptrs.append(warn_d)
            st = _abi.Stack(n=n, width=w, height=h, channels=c, base=dev, frame_stride=stride,
                            frame_offset=frame_offset)
            self.check(lib().cp_composite_device(self.handle, ct.byref(st), ct.byref(p), out_d,
                                                 bl_d, None, warn_d, None),
                       "cp_composite_device")
            self.synchronize()
            out = self.download(out_d, (h, w, c))
            bl = self.download(bl_d, (h, w, c)) if bl_d is not None else None
            warn = int(self.download(warn_d, (1,), np.uint64)[0])
            return out, bl, warn
        finally:
            for q in ptrs:
                self.free(q)

    def composite_multi(self, frames, params_list, blend=True):
        """One host-memory stack under several parameter sets (cp_composite_multi): the
        frames are copied to the device once. Returns [(composite, blend_mask or None,
        warnings)] in the order of params_list."""
        a = _as_stack(frames)
        n, h, w, c = a.shape
        k = len(params_list)
        st = _abi.Stack(n=n, width=w, height=h, channels=c, base=a.ctypes.data,
                        frame_stride=h * w * c)
        ps = (_abi.Params * k)(*params_list)
        outs = [np.empty((h, w, c), dtype=np.uint8) for _ in range(k)]
        bls = [np.empty((h, w, c), dtype=np.uint8) if blend and p.mode == 0 else None
               for p in params_list]
        optr = (ct.c_void_p * k)(*[o.ctypes.data for o in outs])
        bptr = (ct.c_void_p * k)(*[b.ctypes.data if b is not None else None for b in bls])
        warn = (ct.c_uint64 * k)()
        self.check(lib().cp_composite_multi(self.handle, ct.byref(st), ps, k, optr, bptr, warn),
                   "cp_composite_multi")
        return [(outs[i], bls[i], int(warn[i])) for i in range(k)]

    def shake_analyze(self, frames, anchors, anchor_radius, search_radius, diffs=False):
        """ShakeAnalyzer::analyze on the device: per-frame (dx, dy) offsets."""
        a = _as_stack(frames)
        n, h, w, c = a.shape
        ptrs = []
        try:
            for i in range(n):
                ptrs.append(self.upload(a[i]))
            parr = (ct.c_void_p * n)(*ptrs)
            anc = np.ascontiguousarray(np.asarray(anchors, dtype=np.int32).reshape(-1))
            offs = np.zeros((n, 2), np.int32)
            S = 2 * search_radius + 1
            dd = np.zeros((max(n - 1, 0), S, S), np.int32) if diffs else None
            rc = lib().cp_shake_analyze_device(
                self.handle, parr, n, w, h, c, anc.ctypes.data_as(_abi.I32P), len(anc) // 2,
                anchor_radius, search_radius, offs.ctypes.data_as(_abi.I32P),
                dd.ctypes.data_as(_abi.I32P) if dd is not None else None)
            self.check(rc, "cp_shake_analyze_device")
        finally:
            for q in ptrs:
                self.free(q)
        return (offs, dd) if diffs else offs


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx


class OutlierProcessor:
    """OutlierProcessor::new (src/chrono.rs:46-71); process() composites one output frame."""

    def __init__(self, threshold=None, background="random", outlier="extreme",
                 weights=(1.0, 1.0, 1.0, 1.0), fade=None, sample=None, seed=0x5EED,
                 context=None):
        self.kw = dict(mode="outlier", threshold=threshold, background=background,
                       outlier=outlier, weights=weights, fade=fade, sample=sample, seed=seed)
        self.ctx = context

    def process(self, frames, image_indices=None, debug=False):
        """(composite, blend mask) like OutlierProcessor::process (src/chrono.rs:73-206).
        frames: uint8 [n, h, w, c], a sequence of images, or PNG file paths."""
        ctx = self.ctx or default_context()
        a, offset = _select(frames, image_indices)
        r = ctx.composite(a, frame_offset=offset, debug=debug, **self.kw)
        return r if debug else (r[0], r[1])


class SimpleProcessor:
    """SimpleProcessor::new (src/simple.rs:18-24): darker/lighter."""

    def __init__(self, weights=(1.0, 1.0, 1.0, 1.0), fade=None, darker=True, context=None):
        self.kw = dict(mode="darker" if darker else "lighter", weights=weights, fade=fade)
        self.ctx = context

    def process(self, frames, crop=None, image_indices=None):
        ctx = self.ctx or default_context()
        a, offset = _select(frames, image_indices)
        return ctx.composite(a, frame_offset=offset, blend=False, crop=crop, **self.kw)[0]


class Crop:
    """Crop::create (src/shake.rs:136-176) via the library."""

    @staticmethod
    def create(offsets, width, height):
        offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32).reshape(-1))
        n = len(offs) // 2
        has = ct.c_int32(0)
        crops = np.zeros((n, 4), np.int32)
        _check(None, lib().cp_crop_create(offs.ctypes.data_as(_abi.I32P), n, width, height,
                                          ct.byref(has), crops.ctypes.data_as(_abi.I32P)),
               "cp_crop_create")
        return crops if has.value else None


class ShakeAnalyzer:
    def __init__(self, context=None):
        self.ctx = context

    def analyze(self, frames, anchors, anchor_radius, search_radius):
        ctx = self.ctx or default_context()
        return [tuple(o) for o in ctx.shake_analyze(frames, anchors, anchor_radius, search_radius)]


def png_info(path):
    """(width, height, channels) of a PNG file (cp_png_info)."""
    w, h, c = ct.c_int32(), ct.c_int32(), ct.c_int32()
    _check(None, lib().cp_png_info(None, str(path).encode(), ct.byref(w), ct.byref(h),
                                   ct.byref(c)), "cp_png_info")
    return w.value, h.value, c.value


def load_png(paths, threads=0, out=None, context=None):
    """Decodes PNG frames (8-bit gray / RGB / RGBA) on `threads` host threads (0: all) into
    uint8 [n, h, w, c], the layout the compositing entry points take. `out`: optional
    C-contiguous destination of that shape (e.g. pinned memory); the replacement of the
    reference's per-frame `image::open` (src/streams.rs:63-70)."""
    paths = [str(p) for p in paths]
    if not paths:
        raise ValueError("no frames")
    w, h, c = png_info(paths[0])
    if out is None:
        out = np.empty((len(paths), h, w, c), np.uint8)
    if out.shape != (len(paths), h, w, c) or out.dtype != np.uint8 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous uint8 array of shape %s"
                         % ((len(paths), h, w, c),))
    arr = (ct.c_char_p * len(paths))(*[p.encode() for p in paths])
    rc = lib().cp_load_png(context.handle if context else None, arr, len(paths), int(threads),
                           out.ctypes.data, h * w * c, w, h, c)
    _check(context.handle if context else None, rc, "cp_load_png")
    return out


def save_png(path, image, level=6, threads=0, context=None):
    """Writes a uint8 [h, w, c] image (c = 1, 3 or 4) as a PNG file (cp_save_png) on
    `threads` host threads (0: all), creating a missing parent directory like the reference's
    save_image (src/main.rs:519-570)."""
    a = np.ascontiguousarray(image, dtype=np.uint8)
    if a.ndim == 2:
        a = a[:, :, None]
    h, w, c = a.shape
    handle = context.handle if context else None
    _check(handle, lib().cp_save_png(handle, str(path).encode(), a.ctypes.data, w, h, c,
                                     int(level), int(threads)), "cp_save_png")


def jpeg_info(path):
    """(width, height, channels) of a JPEG file (cp_jpeg_info): channels 1 (gray) or 3."""
    w, h, c = ct.c_int32(), ct.c_int32(), ct.c_int32()
    _check(None, lib().cp_jpeg_info(None, str(path).encode(), ct.byref(w), ct.byref(h),
                                    ct.byref(c)), "cp_jpeg_info")
    return w.value, h.value, c.value


def load_jpeg(paths, threads=0, out=None, context=None):
    """Decodes JPEG frames on the GPU (cp_load_jpeg, nvJPEG) into host uint8 [n, h, w, c]
    (c = 3 for colour, 1 for gray), the replacement of the reference's per-frame
    `image::open` (src/streams.rs:63-70). `out`: optional C-contiguous destination of that
    shape (e.g. pinned memory). Context.load_jpeg_device keeps the frames on the device."""
    paths = [str(p) for p in paths]
    if not paths:
        raise ValueError("no frames")
    ctx = context or default_context()
    w, h, c = jpeg_info(paths[0])
    if out is None:
        out = np.empty((len(paths), h, w, c), np.uint8)
    if out.shape != (len(paths), h, w, c) or out.dtype != np.uint8 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous uint8 array of shape %s"
                         % ((len(paths), h, w, c),))
    arr = (ct.c_char_p * len(paths))(*[p.encode() for p in paths])
    ctx.check(lib().cp_load_jpeg(ctx.handle, arr, len(paths), int(threads), out.ctypes.data,
                                 h * w * c, w, h, c), "cp_load_jpeg")
    return out


_SUBSAMPLING = {"444": 0, "4:4:4": 0, "420": 1, "4:2:0": 1}


def encode_jpeg(image, quality=95, subsampling="444", threads=0, context=None):
    """The baseline JPEG bytes of a uint8 [h, w, c] image (cp_encode_jpeg; c = 1, 3 or 4,
    the alpha of 4 dropped), quality 1..100, chroma subsampling "444" (the reference's
    encoder) or "420"."""
    a = np.ascontiguousarray(image, dtype=np.uint8)
    if a.ndim == 2:
        a = a[:, :, None]
    h, w, c = a.shape
    handle = context.handle if context else None
    size = ct.c_uint64(0)
    cap = 1024 + 2 * a.nbytes
    buf = np.empty(cap, np.uint8)
    _check(handle, lib().cp_encode_jpeg(handle, a.ctypes.data, w, h, c, int(quality),
                                        _SUBSAMPLING[subsampling], int(threads),
                                        buf.ctypes.data, cap, ct.byref(size)), "cp_encode_jpeg")
    return buf[:size.value].tobytes()


def save_jpeg(path, image, quality=95, subsampling="444", threads=0, context=None):
    """Writes a uint8 [h, w, c] image as a baseline JPEG file (cp_save_jpeg), creating a
    missing parent directory: the .jpg branch of the reference's save_image
    (src/main.rs:542-556), quality 95 by default as its --quality."""
    a = np.ascontiguousarray(image, dtype=np.uint8)
    if a.ndim == 2:
        a = a[:, :, None]
    h, w, c = a.shape
    handle = context.handle if context else None
    _check(handle, lib().cp_save_jpeg(handle, str(path).encode(), a.ctypes.data, w, h, c,
                                      int(quality), _SUBSAMPLING[subsampling], int(threads)),
           "cp_save_jpeg")


def save_image(path, image, quality=95, threads=0, context=None):
    """save_image of src/main.rs:519-570: JPEG for a .jpg / .jpeg extension (at `quality`),
    PNG otherwise; a missing parent directory is created."""
    if _is_jpeg(path):
        save_jpeg(path, image, quality=quality, threads=threads, context=context)
    elif str(path).lower().endswith(".png"):
        save_png(path, image, threads=threads, context=context)
    else:
        raise ValueError("output format by extension: .png, .jpg or .jpeg")


def sample_indices(n, count, seed=0x5EED):
    """Seeded sub-sample of min(count, n) sorted distinct positions of n frames
    (cp_sample_indices; the reference draws them unseeded, src/chrono.rs:153-158)."""
    out = np.zeros(max(int(n), 1), np.int32)
    got = ct.c_int32(0)
    _check(None, lib().cp_sample_indices(int(n), int(count), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                         out.ctypes.data_as(_abi.I32P), ct.byref(got)),
           "cp_sample_indices")
    return [int(v) for v in out[:got.value]]


def video_windows(image_count, video_in, video_out=(None, None, 1)):
    """chrono-video windows of src/main.rs:230-286: list of (output frame, indices)."""
    (a, b, s), (c, d, t) = video_in, video_out
    nw = ct.c_int32()
    ni = ct.c_int64()
    args = [image_count, a is not None, a or 0, b is not None, b or 0, s or 1,
            c is not None, c or 0, d is not None, d or 0, t or 1]
    _check(None, lib().cp_video_windows(*args, ct.byref(nw), ct.byref(ni), None, None, None,
                                        None), "windows")
    starts = np.zeros(max(nw.value, 1), np.int64)
    lens = np.zeros(max(nw.value, 1), np.int32)
    frames = np.zeros(max(nw.value, 1), np.int32)
    idx = np.zeros(max(ni.value, 1), np.int32)
    _check(None, lib().cp_video_windows(*args, ct.byref(nw), ct.byref(ni),
                                        starts.ctypes.data_as(_abi.I64P),
                                        lens.ctypes.data_as(_abi.I32P),
                                        idx.ctypes.data_as(_abi.I32P),
                                        frames.ctypes.data_as(_abi.I32P)), "windows")
    return [(int(frames[k]), [int(v) for v in idx[starts[k]:starts[k] + lens[k]]])
            for k in range(nw.value)]


class Server:
    """Continuous-batching server (cp_server_*): submit host-memory stacks as they arrive,
    wait for results. Frames given `keys` stay resident on the device and are shared by
    later jobs with the same keys (overlapping chrono-video windows)."""

    def __init__(self, context, hbm_budget=0, max_inflight=8):
        self.ctx = context
        h = ct.c_void_p()
        context.check(lib().cp_server_create(context.handle, hbm_budget, max_inflight,
                                             ct.byref(h)), "cp_server_create")
        self.handle = h
        self.pending = {}

    def submit(self, frames, params=None, keys=None, blend=True, frame_offset=0, **kw):
        """frames: uint8 [n, h, w, c], or a list of n separate C-contiguous [h, w, c] images
        (passed by pointer, not copied; they may repeat)."""
        keep = []
        p = params if params is not None else make_params(keep=keep, **kw)
        job = _abi.Job()
        if isinstance(frames, (list, tuple)) and all(
                isinstance(f, np.ndarray) and f.dtype == np.uint8 and f.flags.c_contiguous
                for f in frames):
            a = list(frames)
            h, w = a[0].shape[:2]
            c = a[0].shape[2] if a[0].ndim == 3 else 1
            n = len(a)
            if any(f.shape != a[0].shape for f in a):
                raise ValueError("frames differ in shape")
            ptrs = (ct.c_void_p * n)(*[f.ctypes.data for f in a])
            keep.append(ptrs)
            job.stack = _abi.Stack(n=n, width=w, height=h, channels=c,
                                   frames=ct.cast(ptrs, ct.POINTER(ct.c_void_p)),
                                   frame_offset=frame_offset)
        else:
            a = _as_stack(frames)
            n, h, w, c = a.shape
            job.stack = _abi.Stack(n=n, width=w, height=h, channels=c, base=a.ctypes.data,
                                   frame_stride=h * w * c, frame_offset=frame_offset)
        if keys is not None:
            karr = (ct.c_uint64 * n)(*[int(k) for k in keys])
            keep.append(karr)
            job.frame_keys = ct.cast(karr, ct.POINTER(ct.c_uint64))
        job.params = p
        out = np.empty((h, w, c), np.uint8)
        bl = np.empty((h, w, c), np.uint8) if blend else None
        job.out = out.ctypes.data
        job.out_blend = bl.ctypes.data if bl is not None else None
        jid = ct.c_uint64()
        self.ctx.check(lib().cp_server_submit(self.handle, ct.byref(job), ct.byref(jid)),
                       "cp_server_submit")
        self.pending[jid.value] = (a, out, bl, keep, p)
        return jid.value

    def wait(self, job_id, timeout_ms=-1):
        r = _abi.JobResult()
        rc = lib().cp_server_wait(self.handle, job_id, timeout_ms, ct.byref(r))
        if rc == _abi.CP_ERR_TIMEOUT:
            return None
        self.ctx.check(rc, "cp_server_wait")
        a, out, bl, keep, p = self.pending.pop(job_id)
        return {"status": r.status, "warnings": r.warnings, "submit_s": r.submit_s,
                "admit_s": r.admit_s, "done_s": r.done_s, "out": out, "blend": bl}

    def cancel(self, job_id):
        """Cancels a job still in the queue: True if cancelled (its wait() then reports status
        CP_ERR_CANCELLED), False if it has already been admitted or has completed."""
        rc = lib().cp_server_cancel(self.handle, job_id)
        if rc == _abi.CP_ERR_STATE:
            return False
        self.ctx.check(rc, "cp_server_cancel")
        return True

    def close(self):
        if self.handle:
            rc = lib().cp_server_destroy(self.handle)
            self.handle = None
            self.ctx.check(rc, "cp_server_destroy")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
