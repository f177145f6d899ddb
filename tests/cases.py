"""Shared helpers of the test suite: parameter construction, random small stacks and
comparisons between the CUDA library, the C++ oracle and the pure-Python restatement."""
import json
import os

import numpy as np

from chrono_photo_gb300 import api

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kat():
    with open(os.path.join(GOLDEN, "kat.json")) as f:
        return json.load(f)


def params(**kw):
    """cp_params plus the ctypes buffers it points into (keep them alive together)."""
    keep = []
    p = api.make_params(keep=keep, **kw)
    p._keep = keep
    return p


def pixel_stack(samples):
    """A 1x1-pixel stack [n, 1, 1, c] from a list of per-frame channel tuples."""
    return np.asarray(samples, dtype=np.uint8).reshape(len(samples), 1, 1, -1)


def random_stack(rng, n, h, w, c, n_spots=3, noise=6):
    """Background with small noise plus bright/dark spots that move over the frames, so
    every mode sees outliers, ties and all-outlier pixels."""
    base = rng.integers(40, 200, size=(1, h, w, c))
    f = base + rng.integers(-noise, noise + 1, size=(n, h, w, c))
    for _ in range(n_spots):
        col = rng.integers(0, 256, size=c)
        for i in range(n):
            if rng.random() < 0.5:
                y, x = rng.integers(0, h), rng.integers(0, w)
                f[i, max(0, y - 1):y + 2, max(0, x - 1):x + 2] = col
    # a few pixels where every frame differs wildly (all outliers under small thresholds)
    f[:, 0, 0] = rng.integers(0, 256, size=(n, c))
    # exact ties
    if n > 2 and h > 1 and w > 1:
        f[:, h - 1, w - 1] = f[0, h - 1, w - 1]
    return np.clip(f, 0, 255).astype(np.uint8)


def assert_close_u8(a, b, tol=1, what=""):
    """Composite/blend parity: within `tol` LSB per band; returns (max, mean) error."""
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    assert d.max() <= tol, "%s: max error %d > %d at %s" % (what, d.max(), tol,
                                                            np.argwhere(d > tol)[:5].tolist())
    return int(d.max()), float(d.mean())
