"""The allocation-free batched entry point, cp_composite_batch_static (needs a GB300).

It exists for callers that cannot call cudaMalloc (a plug-in whose host application's
allocator owns all device memory, a service with a fixed device footprint): its scratch is a
fixed device array inside the library. Its output must equal cp_composite_batch_device's on
the same inputs, and the oracle's, on two calls in a row (the second call finds the previous
call's scratch contents), and its status query must report that every bounded wait
completed. The test allocates its own inputs and outputs; the entry point allocates
nothing."""
import ctypes as ct

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu


def test_static_batch_equals_batch_device(ctx):
    rng = np.random.default_rng(7)
    specs = [(9, 20, 33, dict(mode="outlier", outlier="extreme", background="first")),
             (40, 48, 64, dict(mode="outlier", outlier="forward", background="average",
                               fade="clamp/abs/0,0.2/30,1")),
             (70, 17, 300, dict(mode="outlier", threshold="rel/2/5", outlier="average",
                                background="median")),
             (25, 31, 41, dict(mode="darker"))]
    n_st = len(specs)
    ptrs = []
    keep = []
    try:
        stacks = (_abi.Stack * n_st)()
        params = (_abi.Params * n_st)()
        outs = {k: (ct.c_void_p * n_st)() for k in ("dev", "st")}
        blends = {k: (ct.c_void_p * n_st)() for k in ("dev", "st")}
        shapes = []
        oracle_out = []
        for i, (n, h, w, kw) in enumerate(specs):
            frames = cases.random_stack(rng, n, h, w, 3, n_spots=5)
            base = ctx.upload(frames)
            ptrs.append(base)
            stacks[i] = _abi.Stack(n=n, width=w, height=h, channels=3, base=base,
                                   frame_stride=h * w * 3, frame_offset=i)
            params[i] = cg.make_params(keep=keep, **kw)
            oracle_out.append(oracle.composite(frames, params[i], frame_offset=i))
            for k in ("dev", "st"):
                outs[k][i] = ctx.alloc(h * w * 3)
                blends[k][i] = ctx.alloc(h * w * 3)
                ptrs += [outs[k][i], blends[k][i]]
            shapes.append((h, w, 3))
        warn = {k: ctx.alloc(8 * n_st) for k in ("dev", "st")}
        ptrs += list(warn.values())
        stream = _abi.lib().cp_ctx_stream(ctx.handle)
        ctx.upload(np.zeros(n_st, np.uint64), warn["dev"])
        ctx.check(_abi.lib().cp_composite_batch_device(ctx.handle, stacks, params, n_st,
                                                       outs["dev"], blends["dev"], warn["dev"],
                                                       stream))
        ctx.synchronize()
        ref = [(ctx.download(outs["dev"][i], s), ctx.download(blends["dev"][i], s))
               for i, s in enumerate(shapes)]
        ref_warn = ctx.download(warn["dev"], (n_st,), np.uint64)
        for call in range(2):
            ctx.upload(np.zeros(n_st, np.uint64), warn["st"])
            for i, s in enumerate(shapes):  # stale outputs must be overwritten
                ctx.upload(np.full(s, 77, np.uint8), outs["st"][i])
            rc = _abi.lib().cp_composite_batch_static(stacks, params, n_st, outs["st"],
                                                      blends["st"], warn["st"], stream)
            assert rc == _abi.CP_OK, "call %d: %d" % (call, rc)
            ctx.synchronize()
            status = ct.c_int32(-99)
            assert _abi.lib().cp_composite_batch_static_status(ct.byref(status), stream) == 0
            assert status.value == _abi.CP_OK
            for i, s in enumerate(shapes):
                got = ctx.download(outs["st"][i], s)
                cases.assert_close_u8(got, ref[i][0], what="call %d composite %d" % (call, i))
                cases.assert_close_u8(got, oracle_out[i][0],
                                      what="call %d composite %d vs oracle" % (call, i))
                if specs[i][3]["mode"] == "outlier":
                    gb = ctx.download(blends["st"][i], s)
                    cases.assert_close_u8(gb, ref[i][1], what="call %d blend %d" % (call, i))
                    cases.assert_close_u8(gb, oracle_out[i][1],
                                          what="call %d blend %d vs oracle" % (call, i))
            got_warn = ctx.download(warn["st"], (n_st,), np.uint64)
            assert np.array_equal(got_warn, ref_warn)
            assert [int(x) for x in got_warn] == [o[2] if specs[i][3]["mode"] == "outlier" else 0
                                                  for i, o in enumerate(oracle_out)]
    finally:
        for p in ptrs:
            ctx.free(p)


def test_static_batch_limit(ctx):
    st = (_abi.Stack * 65)()
    pa = (_abi.Params * 65)()
    outs = (ct.c_void_p * 65)()
    assert _abi.lib().cp_composite_batch_static(st, pa, 65, outs, None, None, None) == _abi.CP_ERR_LIMIT


def test_static_batch_replays_from_a_captured_graph(ctx):
    """The call reads no host memory after it returns (the descriptors travel as kernel
    parameters), so it can be captured into a CUDA graph: two replays of the captured call
    give the oracle's composites."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    specs = [(12, 24, 40, dict(mode="outlier", outlier="average", background="first")),
             (36, 16, 72, dict(mode="outlier", threshold="rel/2/5", outlier="backward",
                               background="median"))]
    n_st = len(specs)
    ptrs, keep, shapes, oracle_out = [], [], [], []
    try:
        stacks = (_abi.Stack * n_st)()
        params = (_abi.Params * n_st)()
        outs = (ct.c_void_p * n_st)()
        blends = (ct.c_void_p * n_st)()
        for i, (n, h, w, kw) in enumerate(specs):
            frames = cases.random_stack(rng, n, h, w, 3, n_spots=4)
            base = ctx.upload(frames)
            ptrs.append(base)
            stacks[i] = _abi.Stack(n=n, width=w, height=h, channels=3, base=base,
                                   frame_stride=h * w * 3, frame_offset=0)
            params[i] = cg.make_params(keep=keep, **kw)
            oracle_out.append(oracle.composite(frames, params[i], frame_offset=0))
            outs[i] = ctx.alloc(h * w * 3)
            blends[i] = ctx.alloc(h * w * 3)
            ptrs += [outs[i], blends[i]]
            shapes.append((h, w, 3))
        warn = ctx.alloc(8 * n_st)
        ptrs.append(warn)
        s = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            rc = _abi.lib().cp_composite_batch_static(stacks, params, n_st, outs, blends, warn,
                                                      ct.c_void_p(s.cuda_stream))
        assert rc == _abi.CP_OK
        for replay in range(2):
            ctx.upload(np.zeros(n_st, np.uint64), warn)
            for i, shp in enumerate(shapes):
                ctx.upload(np.full(shp, 77, np.uint8), outs[i])
            g.replay()
            s.synchronize()
            status = ct.c_int32(-99)
            assert _abi.lib().cp_composite_batch_static_status(
                ct.byref(status), ct.c_void_p(s.cuda_stream)) == 0
            assert status.value == _abi.CP_OK
            for i, shp in enumerate(shapes):
                cases.assert_close_u8(ctx.download(outs[i], shp), oracle_out[i][0],
                                      what="replay %d composite %d" % (replay, i))
                cases.assert_close_u8(ctx.download(blends[i], shp), oracle_out[i][1],
                                      what="replay %d blend %d" % (replay, i))
            assert [int(x) for x in ctx.download(warn, (n_st,), np.uint64)] == \
                [o[2] for o in oracle_out]
        del g
    finally:
        for p in ptrs:
            ctx.free(p)
