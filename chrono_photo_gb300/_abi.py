"""ctypes mirror of include/chrono_gpu.h and the loader of libchrono_gpu.so.

The library is loaded from chrono_photo_gb300/lib/ (built in-tree by build.py). There is no
CPU fallback: if the library or an sm_103 device is missing, calls fail loudly.
"""
import ctypes as ct
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("CHRONO_GPU_LIB") or os.path.join(HERE, "lib", "libchrono_gpu.so")

CP_OK = 0
CP_ERR_ARG = -1
CP_ERR_OOM = -2
CP_ERR_TIMEOUT = -3
CP_ERR_CUDA = -4
CP_ERR_BUDGET = -5
CP_ERR_RANGE = -6
CP_ERR_STATE = -7
CP_ERR_NODEV = -8
CP_ERR_LIMIT = -9
CP_ERR_IO = -10
CP_ERR_CANCELLED = -11

MODE = {"outlier": 0, "darker": 1, "lighter": 2}
OUTLIER = {"first": 0, "last": 1, "extreme": 2, "average": 3, "forward": 4, "backward": 5}
BACKGROUND = {"first": 0, "random": 1, "average": 2, "median": 3}
MAX_FRAMES = 128


class Fade(ct.Structure):
    _fields_ = [("enabled", ct.c_int32), ("repeat", ct.c_int32), ("absolute", ct.c_int32),
                ("n_points", ct.c_int32), ("frames", ct.POINTER(ct.c_int32)),
                ("values", ct.POINTER(ct.c_float))]


class Params(ct.Structure):
    _fields_ = [("mode", ct.c_int32), ("thr_abs", ct.c_int32), ("thr_min", ct.c_float),
                ("thr_max", ct.c_float), ("outlier", ct.c_int32), ("background", ct.c_int32),
                ("weights", ct.c_float * 4), ("fade", Fade),
                ("sample", ct.POINTER(ct.c_int32)), ("n_sample", ct.c_int32),
                ("rng_seed", ct.c_uint64)]


class Stack(ct.Structure):
    _fields_ = [("n", ct.c_int32), ("width", ct.c_int32), ("height", ct.c_int32),
                ("channels", ct.c_int32), ("frames", ct.POINTER(ct.c_void_p)),
                ("base", ct.c_void_p), ("frame_stride", ct.c_int64),
                ("crop", ct.POINTER(ct.c_int32)), ("src_width", ct.c_int32),
                ("src_height", ct.c_int32), ("frame_offset", ct.c_int32)]


class Debug(ct.Structure):
    _fields_ = [("median", ct.c_void_p), ("q1", ct.c_void_p), ("q3", ct.c_void_p),
                ("outlier_bits", ct.c_void_p), ("chosen", ct.c_void_p),
                ("background", ct.c_void_p), ("n_outliers", ct.c_void_p)]


class Job(ct.Structure):
    _fields_ = [("stack", Stack), ("frame_keys", ct.POINTER(ct.c_uint64)), ("params", Params),
                ("out", ct.c_void_p), ("out_blend", ct.c_void_p)]


class JobResult(ct.Structure):
    _fields_ = [("status", ct.c_int32), ("warnings", ct.c_uint64), ("submit_s", ct.c_double),
                ("admit_s", ct.c_double), ("done_s", ct.c_double)]


CP_MAX_SETTINGS = 16

P = ct.c_void_p
I32 = ct.c_int32
I32P = ct.POINTER(ct.c_int32)
I64P = ct.POINTER(ct.c_int64)
U64 = ct.c_uint64
U64P = ct.POINTER(ct.c_uint64)

# (name, restype, argtypes) of every entry point declared in include/chrono_gpu.h
SIGNATURES = [
    ("cp_version", ct.c_char_p, []),
    ("cp_status_str", ct.c_char_p, [ct.c_int]),
    ("cp_params_default", None, [ct.POINTER(Params)]),
    ("cp_fade_lut", ct.c_int, [ct.POINTER(Fade), I32, I32, ct.POINTER(ct.c_float)]),
    ("cp_video_windows", ct.c_int, [I32, I32, I32, I32, I32, I32, I32, I32, I32, I32, I32,
                                    I32P, I64P, I64P, I32P, I32P, I32P]),
    ("cp_crop_create", ct.c_int, [I32P, I32, I32, I32, I32P, I32P]),
    ("cp_sample_indices", ct.c_int, [I32, I32, U64, I32P, I32P]),
    ("cp_ctx_create", ct.c_int, [I32, U64, ct.POINTER(P)]),
    ("cp_ctx_destroy", None, [P]),
    ("cp_ctx_last_error", ct.c_int, [P, ct.c_char_p, ct.c_size_t]),
    ("cp_ctx_stream", P, [P]),
    ("cp_ctx_synchronize", ct.c_int, [P]),
    ("cp_ctx_set_wait_limit", ct.c_int, [P, U64]),
    ("cp_ctx_fail_allocations", ct.c_int, [P, I32]),
    ("cp_ctx_tuning_report", ct.c_int, [P, ct.c_char_p, ct.c_size_t]),
    ("cp_dev_alloc", ct.c_int, [P, U64, ct.POINTER(P)]),
    ("cp_dev_free", ct.c_int, [P, P]),
    ("cp_host_alloc", ct.c_int, [P, U64, ct.POINTER(P)]),
    ("cp_host_free", ct.c_int, [P, P]),
    ("cp_memcpy_h2d", ct.c_int, [P, P, P, U64, P]),
    ("cp_memcpy_d2h", ct.c_int, [P, P, P, U64, P]),
    ("cp_composite_device", ct.c_int, [P, ct.POINTER(Stack), ct.POINTER(Params), P, P,
                                       ct.POINTER(Debug), P, P]),
    ("cp_composite", ct.c_int, [P, ct.POINTER(Stack), ct.POINTER(Params), P, P,
                                ct.POINTER(Debug), U64P]),
    ("cp_composite_multi", ct.c_int, [P, ct.POINTER(Stack), ct.POINTER(Params), I32,
                                      ct.POINTER(P), ct.POINTER(P), U64P]),
    ("cp_composite_device_multi", ct.c_int, [P, ct.POINTER(Stack), ct.POINTER(Params), I32,
                                             ct.POINTER(P), ct.POINTER(P), P, P]),
    ("cp_ctx_launch_counts", ct.c_int, [P, U64P, U64P, U64P]),
    ("cp_composite_batch_device", ct.c_int, [P, ct.POINTER(Stack), ct.POINTER(Params), I32,
                                             ct.POINTER(P), ct.POINTER(P), P, P]),
    ("cp_composite_video_device", ct.c_int, [P, ct.POINTER(P), I32, I32, I32, I32, I32, I64P,
                                             I32P, I32P, ct.POINTER(Params), ct.POINTER(P),
                                             ct.POINTER(P), P, P]),
    ("cp_composite_batch_static", ct.c_int, [ct.POINTER(Stack), ct.POINTER(Params), I32,
                                             ct.POINTER(P), ct.POINTER(P), P, P]),
    ("cp_composite_batch_static_status", ct.c_int, [I32P, P]),
    ("cp_shake_analyze_device", ct.c_int, [P, ct.POINTER(P), I32, I32, I32, I32, I32P, I32,
                                           I32, I32, I32P, I32P]),
    ("cp_server_create", ct.c_int, [P, U64, I32, ct.POINTER(P)]),
    ("cp_server_submit", ct.c_int, [P, ct.POINTER(Job), U64P]),
    ("cp_server_wait", ct.c_int, [P, U64, I32, ct.POINTER(JobResult)]),
    ("cp_server_cancel", ct.c_int, [P, U64]),
    ("cp_server_destroy", ct.c_int, [P]),
    ("cp_png_info", ct.c_int, [P, ct.c_char_p, I32P, I32P, I32P]),
    ("cp_load_png", ct.c_int, [P, ct.POINTER(ct.c_char_p), I32, I32, P, U64, I32, I32, I32]),
    ("cp_save_png", ct.c_int, [P, ct.c_char_p, P, I32, I32, I32, I32, I32]),
    ("cp_jpeg_info", ct.c_int, [P, ct.c_char_p, I32P, I32P, I32P]),
    ("cp_load_jpeg", ct.c_int, [P, ct.POINTER(ct.c_char_p), I32, I32, P, U64, I32, I32, I32]),
    ("cp_load_jpeg_device", ct.c_int, [P, ct.POINTER(ct.c_char_p), I32, I32, P, U64, I32, I32,
                                       I32]),
    ("cp_save_jpeg", ct.c_int, [P, ct.c_char_p, P, I32, I32, I32, I32, I32, I32]),
    ("cp_encode_jpeg", ct.c_int, [P, P, I32, I32, I32, I32, I32, I32, P, U64,
                                  ct.POINTER(ct.c_uint64)]),
]

_lib = None


class ChronoError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        super().__init__("%s (%d)%s" % (STATUS_NAMES.get(status, "error"), status,
                                        ": " + message if message else ""))


STATUS_NAMES = {CP_OK: "ok", CP_ERR_ARG: "invalid argument", CP_ERR_OOM: "out of memory",
                CP_ERR_TIMEOUT: "timed out", CP_ERR_CUDA: "CUDA error",
                CP_ERR_BUDGET: "HBM budget exceeded", CP_ERR_RANGE: "out of range",
                CP_ERR_STATE: "invalid state", CP_ERR_NODEV: "no sm_103 device",
                CP_ERR_LIMIT: "above a fixed limit", CP_ERR_IO: "image file error",
                CP_ERR_CANCELLED: "cancelled"}


def lib():
    """The loaded libchrono_gpu.so with every prototype set (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libchrono_gpu.so is not built (run __graft_entry__.build()): %s"
                          % LIB_PATH)
        l = ct.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib
