"""GB300-native frame-stack compositing for chrono-photo's hot path.

The product is libchrono_gpu.so (include/chrono_gpu.h): hand-written sm_103a kernels behind a
C ABI. This package builds it in-tree (build.py), binds it with ctypes (_abi.py) and mirrors
the reference's processor interface in Python (api.py).
"""
from ._abi import ChronoError, lib  # noqa: F401
from .api import (Context, Crop, Fade, OutlierProcessor, Server, ShakeAnalyzer,  # noqa: F401
                  SimpleProcessor, Threshold, default_context, encode_jpeg, jpeg_info,
                  load_jpeg, load_png, make_params, png_info, save_image, save_jpeg, save_png,
                  video_windows)
