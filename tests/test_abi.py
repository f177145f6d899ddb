"""The C ABI boundary on the CPU: the library loads, exports every entry point of
include/chrono_gpu.h, and its host-only helpers agree with the oracle. No kernel runs."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle, pyref
from tests import cases

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "chrono_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cp_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "cp_composite" in names and "cp_composite_batch_device" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = ct.CDLL(_abi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    bound = {n for n, _, _ in _abi.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_struct_sizes_match_c_layout():
    # cp_params: 6*4 + 16 + cp_fade(4*4 + 2*8) + 8 + 4 (+4 pad) + 8
    assert ct.sizeof(_abi.Fade) == 32
    assert ct.sizeof(_abi.Params) == 24 + 16 + 32 + 8 + 8 + 8
    assert ct.sizeof(_abi.Stack) == 16 + 8 + 8 + 8 + 8 + 16


def test_oracle_structs_match_binding():
    """The oracle's own copies of the C layouts (it imports nothing of the product) match the
    product binding field by field: same names, types, offsets and sizes."""
    for a, b in ((oracle.Fade, _abi.Fade), (oracle.Params, _abi.Params),
                 (oracle.Stack, _abi.Stack), (oracle.Debug, _abi.Debug)):
        assert ct.sizeof(a) == ct.sizeof(b)
        assert [f for f, _ in a._fields_] == [f for f, _ in b._fields_]
        for (name, _), _x in zip(a._fields_, b._fields_):
            assert getattr(a, name).offset == getattr(b, name).offset
            assert getattr(a, name).size == getattr(b, name).size


@pytest.mark.parametrize("kw", [dict(), dict(mode="darker"), dict(mode="lighter", weights=(1, 0.5)),
                                dict(threshold="rel/3/6", outlier="average", background="first"),
                                dict(threshold="abs/0.1", fade="clamp/rel/0,1/4,0", weights=(1, 0, 2)),
                                dict(sample=[0, 2, 5], seed=7, outlier="backward")])
def test_oracle_params_match_make_params(kw):
    """oracle.params (pure Python, used by the benchmark's reference arm) builds the same
    cp_params as the product's make_params; pointer fields are compared by what they hold."""
    a = oracle.params(**kw)
    b = cases.params(**kw)

    def strip(p):
        q = oracle.Params.from_buffer_copy(bytes(p))
        q.fade.frames = None
        q.fade.values = None
        q.sample = None
        return bytes(q)
    assert strip(a) == strip(b)
    n = a.fade.n_points
    assert [a.fade.frames[i] for i in range(n)] == [b.fade.frames[i] for i in range(n)]
    assert [a.fade.values[i] for i in range(n)] == [b.fade.values[i] for i in range(n)]
    assert [a.sample[i] for i in range(a.n_sample)] == [b.sample[i] for i in range(b.n_sample)]


def test_version_and_status():
    lib = cg.lib()
    assert b"sm_103a" in lib.cp_version()
    assert lib.cp_status_str(-6) == b"coordinate out of range"


def test_params_default_match_cli_defaults():
    p = _abi.Params()
    cg.lib().cp_params_default(ct.byref(p))
    # src/cli.rs:192-216
    assert (p.mode, p.thr_abs, p.outlier, p.background) == (0, 1, 2, 1)
    assert abs(p.thr_min - 0.05) < 1e-7 and abs(p.thr_max - 0.2) < 1e-7
    assert list(p.weights) == [1.0, 1.0, 1.0, 1.0] and p.fade.enabled == 0


@pytest.mark.parametrize("spec,n,offset", [("clamp/abs/0,0/10,1", 12, 0), ("repeat/abs/0,1/5,0", 17, 3),
                                          ("clamp/rel/0,1/4,0", 9, 0), ("repeat/rel/-2,0.5/1,1/3,0", 11, 5),
                                          ("clamp/abs/3,0.25/4,2", 10, 2)])
def test_fade_lut_matches_reference(spec, n, offset):
    fd = cg.Fade.parse(spec)
    got = fd.lut(n, offset)
    f = pyref.fade_table(fd.repeat, fd.absolute, fd.points)
    want = np.array([f(i, n, offset) for i in range(n)], np.float32)
    assert np.array_equal(got, want)
    keep = []
    c = fd.to_c(keep)
    assert np.array_equal(oracle.fade_lut(c, n, offset), want)


def test_video_windows_match_oracle():
    rng = np.random.default_rng(1)
    for _ in range(200):
        count = int(rng.integers(1, 40))
        s = int(rng.integers(-5, 10)) if rng.random() < 0.8 else None
        e = (s if s is not None else 0) + int(rng.integers(1, 12)) if rng.random() < 0.8 else None
        step = int(rng.integers(1, 4))
        vo = (int(rng.integers(-8, 4)) if rng.random() < 0.3 else None,
              int(rng.integers(5, 40)) if rng.random() < 0.3 else None, int(rng.integers(1, 3)))
        assert cg.video_windows(count, (s, e, step), vo) == oracle.video_windows(count, (s, e, step), vo)


def test_crop_matches_oracle():
    rng = np.random.default_rng(2)
    for _ in range(50):
        offs = rng.integers(-12, 13, size=(int(rng.integers(1, 9)), 2))
        offs[0] = 0
        a = cg.Crop.create(offs, 640, 480)
        b = oracle.crop_create(offs, 640, 480)
        assert (a is None and b is None) or np.array_equal(a, b)


def test_sample_indices_sorted_distinct():
    out = (ct.c_int32 * 64)()
    n = ct.c_int32()
    assert cg.lib().cp_sample_indices(64, 20, 7, out, ct.byref(n)) == 0
    v = list(out)[: n.value]
    assert n.value == 20 and v == sorted(set(v)) and all(0 <= x < 64 for x in v)
    assert cg.lib().cp_sample_indices(10, 20, 7, out, ct.byref(n)) == 0 and n.value == 10


def test_invalid_args_without_device():
    lib = cg.lib()
    assert lib.cp_composite(None, None, None, None, None, None, None) == _abi.CP_ERR_ARG
    assert lib.cp_ctx_create(0, 0, None) == _abi.CP_ERR_ARG
    w = ct.c_int32()
    i = ct.c_int64()
    assert lib.cp_video_windows(10, 1, 0, 1, 5, 0, 0, 0, 0, 0, 1, ct.byref(w), ct.byref(i),
                                None, None, None, None) == _abi.CP_ERR_ARG
    # the host-staged multi-setting call checks its arguments before any device work
    st = _abi.Stack(n=4, width=8, height=8, channels=3, base=None, frame_stride=192)
    ps = (_abi.Params * 2)()
    outs = (ct.c_void_p * 2)()
    assert lib.cp_composite_multi(None, ct.byref(st), ps, 2, outs, None, None) == _abi.CP_ERR_ARG
    # frame ingest and output encode need no device at all
    assert lib.cp_load_png(None, None, 1, 0, None, 0, 1, 1, 3) == _abi.CP_ERR_ARG
    assert lib.cp_save_png(None, b"x.png", None, 1, 1, 3, 6, 0) == _abi.CP_ERR_ARG
    h, wd, c = ct.c_int32(), ct.c_int32(), ct.c_int32()
    assert lib.cp_png_info(None, None, ct.byref(wd), ct.byref(h), ct.byref(c)) == _abi.CP_ERR_ARG


def test_context_requires_gpu():
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(cg.ChronoError) as e:
        cg.Context(0)
    assert e.value.status == _abi.CP_ERR_NODEV
