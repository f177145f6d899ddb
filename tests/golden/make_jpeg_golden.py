"""Writes tests/golden/jpeg_golden.npz: small JPEG files made by the library's encoder
(cp_encode_jpeg) and the same files decoded by nvJPEG on a GB300 (cp_load_jpeg), the
third-party decoder the product ingests frames with, by both of its routes. The CPU tests hold the oracle's
exact-IDCT decoder to these decodings (and the encoder to these bytes).

Run on a machine with the GPU, from the repository root:
    python tests/golden/make_jpeg_golden.py [output.npz]
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import chrono_photo_gb300 as cg  # noqa: E402


def image(h, w, c, seed, noise=4.0):
    """A seeded gradient with Gaussian noise and a dark disk (channels 1, 3 or 4)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    a = np.stack([255 * x / max(w - 1, 1), 255 * y / max(h - 1, 1),
                  127 * (x + y) / max(w + h - 2, 1) + 64], -1)
    a[(x - w / 3) ** 2 + (y - h / 2) ** 2 < (min(h, w) / 4) ** 2] *= 0.2
    a += rng.normal(0, noise, a.shape)
    a = np.clip(np.rint(a), 0, 255).astype(np.uint8)
    if c == 1:
        return a[..., :1]
    if c == 4:
        return np.concatenate([a, np.full((h, w, 1), 255, np.uint8)], -1)
    return a


# (name, height, width, channels, quality, subsampling, seed)
CASES = [("rgb444_q95", 48, 64, 3, 95, "444", 1),
         ("rgb444_q75_odd", 37, 53, 3, 75, "444", 2),
         ("rgb420_q90", 48, 64, 3, 90, "420", 3),
         ("rgb420_q60_odd", 41, 29, 3, 60, "420", 4),
         ("gray_q95", 40, 56, 1, 95, "444", 5)]


def main(out):
    """Per case: the source image, the JPEG bytes, and nvJPEG's decoding by the GPU's JPEG
    engines ("engine", the default route) and by its software backend ("software",
    CP_JPEG_BACKEND=default)."""
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        paths = {}
        for name, h, w, c, q, ss, seed in CASES:
            src = image(h, w, c, seed)
            data = cg.encode_jpeg(src, quality=q, subsampling=ss)
            paths[name] = os.path.join(tmp, name + ".jpg")
            with open(paths[name], "wb") as f:
                f.write(data)
            arrays[name + "/source"] = src
            arrays[name + "/jpeg"] = np.frombuffer(data, np.uint8)
        for route, env in (("engine", None), ("software", "default")):
            if env:
                os.environ["CP_JPEG_BACKEND"] = env
            else:
                os.environ.pop("CP_JPEG_BACKEND", None)
            with cg.Context(0) as ctx:  # the backend is chosen at the context's first decode
                for name in paths:
                    arrays[name + "/" + route] = cg.load_jpeg([paths[name]], context=ctx)[0]
        os.environ.pop("CP_JPEG_BACKEND", None)
    np.savez_compressed(out, **arrays)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden",
                                                              "jpeg_golden.npz"))
