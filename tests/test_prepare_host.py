"""Option semantics on the host, without a GPU: the descriptor fields prepare_stack
(csrc/cp_prepare.cpp) derives from a stack and its options, read through the test hook of the
CPU-built host library (tests/mock_device, mock_prepare).

- the median and quartile positions reproduce the reference's median() and quantile()
  (src/chrono.rs:567-591) on sorted samples, in f32, through the kernels' quantile formula;
- the integer threshold table is the smallest D' with D' + nh/4 >= thr^2 (abs thresholds with
  0/1 weights take exact integer distances);
- fade flags, distance kinds and the errors the reference reports by panicking.
"""
import ctypes as ct
from fractions import Fraction

import numpy as np
import pytest

from chrono_photo_gb300 import _abi, api
from oracle import pyref

F = np.float32


@pytest.fixture(scope="module")
def lib(mock_device_lib):
    return mock_device_lib


def prepare(lib, n, **kw):
    """(status, ints dict, floats dict, fade list) of prepare_stack for an n-frame 8x8 RGB
    stack under make_params(**kw)."""
    keep = []
    p = api.make_params(keep=keep, **kw)
    st = _abi.Stack(n=n, width=8, height=8, channels=3, base=256, frame_stride=8 * 8 * 3)
    ints = (ct.c_int32 * 32)()
    floats = (ct.c_float * (8 + n))()
    rc = lib.mock_prepare(ct.byref(st), ct.byref(p), ints, floats)
    names = ("n", "nw", "n_sub", "med_k", "med_pair", "q1_k", "q1_pair", "q3_k", "q3_pair",
             "fast_int", "pair_f32", "no_fade", "unit_fade", "wmask", "thr_abs")
    iv = dict(zip(names, ints[:15]))
    iv["thr_int"] = list(ints[15:20])
    fv = dict(zip(("q1_frac", "q3_frac", "thr_min", "thr_max", "thr_scale", "thr_sq"),
                  [F(x) for x in floats[:6]]))
    return rc, iv, fv, [F(x) for x in floats[6:6 + n]]


def quantile_value(lo, hi, pair, frac):
    """The kernels' quantile from its order statistics: (1 - frac) * d[k] + frac * d[k+1]
    in f32, or d[k] alone."""
    if not pair:
        return F(lo)
    return F(F(F(F(1) - frac) * F(lo)) + F(frac * F(hi)))


@pytest.mark.parametrize("n", list(range(3, 129)))
def test_order_statistic_positions(lib, n):
    rc, iv, fv, _ = prepare(lib, n, threshold="rel/3/6")
    assert rc == _abi.CP_OK
    assert iv["n_sub"] == n and iv["nw"] == (1 if n <= 32 else 2 if n <= 64 else 4)
    rng = np.random.default_rng(n)
    for _ in range(20):
        d = sorted(int(v) for v in rng.integers(0, 256, n))
        lo, hi = d[iv["med_k"]], d[iv["med_k"] + iv["med_pair"]]
        med = F(F(0.5) * F(F(lo) + F(hi))) if iv["med_pair"] else F(lo)
        assert med == pyref.median(d)
        for q, key in ((0.25, "q1"), (0.75, "q3")):
            k, pair = iv[key + "_k"], iv[key + "_pair"]
            got = quantile_value(d[k], d[k + 1] if pair else d[k], pair, fv[key + "_frac"])
            assert got == pyref.quantile(d, q), (n, q)


def test_subsample_positions(lib):
    """--sample: the positions refer to the sample's own length."""
    for m in (3, 8, 13, 40):
        idx = list(range(0, 2 * m, 2))
        rc, iv, _, _ = prepare(lib, 2 * m, threshold="rel/3/6", sample=idx)
        assert rc == _abi.CP_OK and iv["n_sub"] == m
        rc0, iv0, _, _ = prepare(lib, m, threshold="rel/3/6")
        for key in ("med_k", "med_pair", "q1_k", "q1_pair", "q3_k", "q3_pair"):
            assert iv[key] == iv0[key], (m, key)


@pytest.mark.parametrize("lo", [0.0, 0.01, 0.02, 0.05, 0.0517, 0.1, 0.2, 0.5, 0.999, 1.0])
def test_integer_threshold_table(lib, lo):
    rc, iv, fv, _ = prepare(lib, 16, threshold="abs/%r/%r" % (lo, max(lo, 0.3)))
    assert rc == _abi.CP_OK and iv["fast_int"] == 1 and iv["thr_abs"] == 1
    thr_min = F(F(lo) * F(255))
    assert fv["thr_min"] == thr_min and fv["thr_sq"] == F(thr_min * thr_min)
    thr_sq = Fraction(float(fv["thr_sq"]))
    for nh in range(5):
        t = iv["thr_int"][nh]
        assert t >= 0
        assert Fraction(t) + Fraction(nh, 4) >= thr_sq
        assert t == 0 or Fraction(t - 1) + Fraction(nh, 4) < thr_sq


def test_fade_flags(lib):
    rc, iv, _, fade = prepare(lib, 12)
    assert rc == _abi.CP_OK and iv["no_fade"] == 1 and iv["unit_fade"] == 1
    assert all(f == 1 for f in fade)
    rc, iv, _, fade = prepare(lib, 12, fade="clamp/abs/0,1/10,1")
    assert iv["unit_fade"] == 1 and iv["no_fade"] == 1
    rc, iv, _, fade = prepare(lib, 12, fade="clamp/abs/0,0.5/10,1")
    assert iv["unit_fade"] == 0 and iv["no_fade"] == 0 and fade[0] == F(0.5)
    rc, iv, _, fade = prepare(lib, 12, fade="clamp/abs/0,1/10,2")
    assert iv["unit_fade"] == 0 and iv["no_fade"] == 1 and fade[-1] == F(2)


def test_distance_kinds(lib):
    _, iv, _, _ = prepare(lib, 16, threshold="abs/0.05/0.2")
    assert iv["fast_int"] == 1
    _, iv, _, _ = prepare(lib, 16, threshold="abs/0.05/0.2", weights=[1, 0, 1, 1])
    assert iv["fast_int"] == 1 and iv["wmask"] & 7 == 0b101
    _, iv, _, _ = prepare(lib, 16, threshold="abs/0.05/0.2", weights=[0.5, 2, 1, 1])
    assert iv["fast_int"] == 0 and iv["pair_f32"] == 1
    _, iv, _, _ = prepare(lib, 16, threshold="rel/3/6")
    assert iv["fast_int"] == 0 and iv["pair_f32"] == 1
    _, iv, _, _ = prepare(lib, 16, threshold="rel/3/6", weights=[1, -1, 1, 1])
    assert iv["fast_int"] == 0 and iv["pair_f32"] == 0  # cancelling sums: scalar f32


def test_errors_the_reference_panics_on(lib):
    assert prepare(lib, 2, threshold="rel/3/6")[0] == _abi.CP_ERR_ARG  # quartiles of 2
    assert prepare(lib, 16, threshold="rel/3/6", sample=[3, 1, 2])[0] == _abi.CP_ERR_ARG
    assert prepare(lib, 16, mode="outlier", sample=[0, 1, 16])[0] == _abi.CP_ERR_ARG
