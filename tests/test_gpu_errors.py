"""Device-side waits that give up (needs a GB300).

Every compositing kernel waits for its staged frame rows on an mbarrier with a bounded wait
(cp_ctx_set_wait_limit). A limit of 1 cycle makes every such wait give up at once: the CTAs
leave once their copies in flight have landed, the call reports CP_ERR_TIMEOUT (host-memory
entry points at once, device entry points at the next cp_ctx_synchronize), and the context
stays usable: with the default limit the same call then matches the oracle. No GPU fault,
trap or hang is involved; the reference has no device side (it panics on I/O errors,
src/chrono.rs:126)."""
import ctypes as ct

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

SETTINGS = [
    ("pixel-thread kernel", 3, dict(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                                    background="first")),
    ("pixel-thread kernel, rel", 3, dict(mode="outlier", threshold="rel/2/4", outlier="average",
                                         background="first")),
    ("tile kernel (one channel)", 1, dict(mode="outlier", threshold="abs/0.05/0.2",
                                          outlier="forward", background="median")),
    ("streaming darker kernel", 3, dict(mode="darker")),
]


@pytest.mark.parametrize("name,c,kw", SETTINGS, ids=[s[0] for s in SETTINGS])
def test_wait_gives_up_and_context_recovers(ctx, name, c, kw):
    rng = np.random.default_rng(3)
    frames = cases.random_stack(rng, 24, 40, 64, c, n_spots=4)
    p = cases.params(**kw)
    lib = _abi.lib()
    assert lib.cp_ctx_set_wait_limit(ctx.handle, 1) == _abi.CP_OK
    try:
        with pytest.raises(cg.ChronoError) as e:
            ctx.composite(frames, p)
        assert e.value.status == _abi.CP_ERR_TIMEOUT
        # the device entry point reports it at the next synchronize
        n, h, w, _ = frames.shape
        base = ctx.upload(frames)
        out = ctx.alloc(h * w * c)
        try:
            st = _abi.Stack(n=n, width=w, height=h, channels=c, base=base, frame_stride=h * w * c)
            assert lib.cp_composite_device(ctx.handle, ct.byref(st), ct.byref(p), out, None, None,
                                           None, None) == _abi.CP_OK
            assert lib.cp_ctx_synchronize(ctx.handle) == _abi.CP_ERR_TIMEOUT
            assert lib.cp_ctx_synchronize(ctx.handle) == _abi.CP_OK  # the flag was cleared
        finally:
            ctx.free(base)
            ctx.free(out)
    finally:
        assert lib.cp_ctx_set_wait_limit(ctx.handle, 0) == _abi.CP_OK
    got = ctx.composite(frames, p)
    ref = oracle.composite(frames, p)
    cases.assert_close_u8(got[0], ref[0], what=name)
    if kw["mode"] == "outlier":
        cases.assert_close_u8(got[1], ref[1], what=name + " blend")


def test_wait_limit_arguments(ctx):
    lib = _abi.lib()
    assert lib.cp_ctx_set_wait_limit(None, 5) == _abi.CP_ERR_ARG
    assert lib.cp_ctx_set_wait_limit(ctx.handle, 1 << 63) == _abi.CP_ERR_ARG
    assert lib.cp_ctx_set_wait_limit(ctx.handle, 0) == _abi.CP_OK


def test_injected_allocation_failure(ctx):
    """A host-memory composite whose staging allocation fails reports CP_ERR_OOM, device and
    pinned allocations fail the same way, and the next call on the same context succeeds
    (the context's buffers are grown again on demand). A fresh context: its staging buffers
    do not exist yet, so the composite has to allocate."""
    rng = np.random.default_rng(4)
    frames = cases.random_stack(rng, 30, 60, 80, 3, n_spots=4)
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                     background="first")
    lib = _abi.lib()
    with cg.Context(0) as c2:
        assert lib.cp_ctx_fail_allocations(c2.handle, 1) == _abi.CP_OK
        try:
            with pytest.raises(cg.ChronoError) as e:
                c2.composite(frames, p)
            assert e.value.status == _abi.CP_ERR_OOM
            assert lib.cp_ctx_fail_allocations(c2.handle, 2) == _abi.CP_OK
            with pytest.raises(cg.ChronoError) as e:
                c2.alloc(1024)
            assert e.value.status == _abi.CP_ERR_OOM
            ptr = ct.c_void_p()
            assert lib.cp_host_alloc(c2.handle, 4096, ct.byref(ptr)) == _abi.CP_ERR_OOM
        finally:
            assert lib.cp_ctx_fail_allocations(c2.handle, 0) == _abi.CP_OK
        assert lib.cp_ctx_fail_allocations(c2.handle, -1) == _abi.CP_ERR_ARG
        got = c2.composite(frames, p)
    ref = oracle.composite(frames, p)
    cases.assert_close_u8(got[0], ref[0], what="after an injected failure")
