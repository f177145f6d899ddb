"""The compositing server's queue, admission, cancel and failure handling, on the CPU.

The real server (csrc/cp_server.cpp), option preparation (cp_prepare.cpp) and memory accounting
(cp_memory.cpp) are compiled with g++ against a host-memory stand-in for the CUDA runtime and
for the batched launch (tests/mock_device). Its "device" is a host thread that runs each
stream's queue in order; the tests hold uploads, kernels or downloads to pin the server in a
state, make a launch report a device-side wait that gave up, raise a sticky device fault, and
make allocations fail. The mock kernel writes, per job, the byte-wise max of the frames to the
composite and the min to the blend mask, and counts n warnings, so each job's results show
that its own frames, outputs and counters went through. The GPU tests (test_gpu_server.py)
cover the same server with the real kernels.

Reference behaviour this serves: chrono-photo composites one output at a time and stops at the
first error (src/main.rs:22-211); the server keeps that per-output result, and an error of one
job (a failed allocation, a device-side wait that gave up) fails that job only.
"""
import ctypes as ct
import threading
import time

import numpy as np
import pytest

from chrono_photo_gb300 import _abi

STATS = ("uploads", "upload_bytes", "downloads", "launches", "launches_run", "live_events",
         "live_streams", "live_pools", "pool_bytes", "live_host", "live_dev", "misuse",
         "max_pending", "stacks", "max_stacks")
HOLD_UPLOADS, HOLD_KERNELS, HOLD_DOWNLOADS = 1, 2, 4
POOL, MALLOC, HOSTALLOC = 1, 2, 4

P, U64, I32 = ct.c_void_p, ct.c_uint64, ct.c_int32


@pytest.fixture(scope="module")
def mock(mock_device_lib):
    lib = mock_device_lib
    yield lib
    lib.mock_shutdown()


@pytest.fixture
def dev(mock):
    mock.mock_reset()
    yield mock


def stats(lib):
    buf = (U64 * len(STATS))()
    lib.mock_stats(buf, len(STATS))
    return dict(zip(STATS, buf))


def frame_uploads(lib):
    """Host->device copies of frames (each launch also uploads its descriptors)."""
    s = stats(lib)
    return s["uploads"] - s["launches"]


def poll(cond, timeout=10.0):
    end = time.time() + timeout
    while time.time() < end:
        if cond():
            return True
        time.sleep(0.002)
    return cond()


def frames_for(n, h=6, w=10, c=3, seed=0):
    return np.random.default_rng(seed).integers(0, 256, (n, h, w, c), dtype=np.uint8)


class Server:
    """A server on a mock context; keeps every submitted job's buffers alive until waited."""

    def __init__(self, lib, ctx_budget=0, budget=0, inflight=4):
        self.lib = lib
        self.ctx = lib.mock_ctx_create(ctx_budget)
        h = P()
        assert lib.cp_server_create(self.ctx, budget, inflight, ct.byref(h)) == _abi.CP_OK
        self.h = h
        self.jobs = {}

    def submit(self, frames, keys=None, blend=True, **opt):
        n, hgt, wid, c = frames.shape
        frames = np.ascontiguousarray(frames)
        params = _abi.Params()
        self.lib.cp_params_default(ct.byref(params))
        for k, v in opt.items():
            setattr(params, k, v)
        job = _abi.Job()
        job.params = params
        job.stack.n, job.stack.width, job.stack.height, job.stack.channels = n, wid, hgt, c
        job.stack.base = frames.ctypes.data
        job.stack.frame_stride = hgt * wid * c
        out = np.full((hgt, wid, c), 7, np.uint8)
        bl = np.full((hgt, wid, c), 7, np.uint8) if blend else None
        job.out = out.ctypes.data
        job.out_blend = bl.ctypes.data if blend else None
        karr = None
        if keys is not None:
            karr = (U64 * n)(*keys)
            job.frame_keys = karr
        jid = U64()
        rc = self.lib.cp_server_submit(self.h, ct.byref(job), ct.byref(jid))
        if rc == _abi.CP_OK:
            self.jobs[jid.value] = (frames, out, bl, karr)
        return rc, jid.value

    def wait(self, jid, timeout_ms=10000):
        res = _abi.JobResult()
        rc = self.lib.cp_server_wait(self.h, jid, timeout_ms, ct.byref(res))
        if rc != _abi.CP_OK:
            return rc, None, None, None
        frames, out, bl, _ = self.jobs.pop(jid)
        return rc, res, out, bl

    def check_ok(self, jid):
        frames = self.jobs[jid][0]
        rc, res, out, bl = self.wait(jid)
        assert rc == _abi.CP_OK and res.status == _abi.CP_OK, (rc, res and res.status)
        np.testing.assert_array_equal(out, frames.max(axis=0))
        if bl is not None:
            np.testing.assert_array_equal(bl, frames.min(axis=0))
        assert res.warnings == frames.shape[0]
        assert res.submit_s <= res.admit_s <= res.done_s
        return res

    def last_error(self):
        buf = ct.create_string_buffer(512)
        self.lib.cp_ctx_last_error(self.ctx, buf, 512)
        return buf.value.decode()

    def close(self):
        rc = self.lib.cp_server_destroy(self.h)
        used = self.lib.mock_ctx_used(self.ctx)
        self.lib.mock_ctx_destroy(self.ctx)
        return rc, used


def assert_clean(lib, used):
    """Nothing left behind once the server is destroyed and its frees have run."""
    assert used == 0
    assert lib.mock_wait_idle(5000) == 0
    s = stats(lib)
    for k in ("live_events", "live_streams", "live_pools", "pool_bytes", "live_host",
              "live_dev", "misuse"):
        assert s[k] == 0, (k, s)


def test_jobs_of_every_shape_complete_with_their_own_results(dev):
    srv = Server(dev, inflight=16)
    ids = []
    for i, (c, n) in enumerate((c, n) for c in (1, 3, 4) for n in (1, 5, 40, 70)):
        rc, jid = srv.submit(frames_for(n, c=c, seed=i), blend=(i % 2 == 0))
        assert rc == _abi.CP_OK
        ids.append(jid)
    for jid in ids:
        srv.check_ok(jid)
    s = stats(dev)
    assert s["launches"] == s["launches_run"] >= 9  # 3 channel counts x 3 plane-word groups
    assert dev.mock_ctx_launches(srv.ctx) == s["launches"]
    assert_clean(dev, srv.close()[1])


def test_cancel_queued_job_and_refuse_admitted_one(dev):
    srv = Server(dev, inflight=1)
    dev.mock_hold(HOLD_UPLOADS)
    fa, fb, fc = frames_for(4, seed=1), frames_for(4, seed=2), frames_for(4, seed=3)
    a, b, c = (srv.submit(f)[1] for f in (fa, fb, fc))
    assert poll(lambda: stats(dev)["uploads"] >= 4)  # a admitted, its uploads held
    assert dev.cp_server_cancel(srv.h, b) == _abi.CP_OK
    assert dev.cp_server_cancel(srv.h, a) == _abi.CP_ERR_STATE  # admitted: runs to the end
    assert dev.cp_server_cancel(srv.h, 12345) == _abi.CP_ERR_ARG
    rc, res, out, _ = srv.wait(b, 1000)
    assert rc == _abi.CP_OK and res.status == _abi.CP_ERR_CANCELLED
    assert (out == 7).all()  # a cancelled job's buffers are not touched
    assert srv.wait(a, 50)[0] == _abi.CP_ERR_TIMEOUT  # held: not done yet
    assert srv.wait(a, 0)[0] == _abi.CP_ERR_TIMEOUT
    dev.mock_hold(0)
    srv.check_ok(a)
    srv.check_ok(c)
    assert dev.cp_server_cancel(srv.h, a) == _abi.CP_ERR_ARG  # collected
    assert srv.wait(b, 0)[0] == _abi.CP_ERR_STATE
    assert frame_uploads(dev) == 8  # b's frames were never uploaded
    assert_clean(dev, srv.close()[1])


def test_injected_allocation_failures_fail_only_their_jobs(dev):
    srv = Server(dev, inflight=1)
    assert dev.cp_ctx_fail_allocations(srv.ctx, 3) == _abi.CP_OK
    ids = [srv.submit(frames_for(5, seed=i))[1] for i in range(4)]
    for jid in ids[:3]:
        rc, res, out, _ = srv.wait(jid)
        assert rc == _abi.CP_OK and res.status == _abi.CP_ERR_OOM
        assert (out == 7).all()
    assert "injected" in srv.last_error()
    srv.check_ok(ids[3])
    assert_clean(dev, srv.close()[1])


@pytest.mark.parametrize("k", [0, 1, 2, 4, 5])
def test_pool_exhausted_at_each_allocation_of_admission(dev, k):
    """The k-th device allocation of a 5-frame job fails (k = 5: the outputs): the job fails
    with CP_ERR_OOM, what it had allocated is returned, and the next job runs."""
    n, h, w, c = 5, 6, 10, 3
    fbytes = h * w * c
    pitch = (fbytes + 16 + 255) // 256 * 256
    srv = Server(dev, inflight=1)
    dev.mock_set_pool_limit(k * pitch + pitch - 1)
    rc, jid = srv.submit(frames_for(n, h, w, c))
    rc, res, _, _ = srv.wait(jid)
    assert rc == _abi.CP_OK and res.status == _abi.CP_ERR_OOM
    assert "cudaMallocFromPoolAsync" in srv.last_error()
    assert dev.mock_ctx_used(srv.ctx) == 0  # no launch yet: nothing else holds memory
    assert poll(lambda: stats(dev)["pool_bytes"] == 0)
    dev.mock_set_pool_limit(0)
    srv.check_ok(srv.submit(frames_for(n, h, w, c, seed=9))[1])
    assert_clean(dev, srv.close()[1])


@pytest.mark.parametrize("kind", [HOSTALLOC, MALLOC])
def test_staging_and_launch_slot_allocation_failures(dev, kind):
    """A pinned staging buffer (admission) or a launch slot's descriptor memory that cannot
    be allocated fails the jobs that needed it with CP_ERR_OOM; later jobs run."""
    srv = Server(dev, inflight=4)
    dev.mock_fail_allocs(kind, 1)
    rc, jid = srv.submit(frames_for(3, seed=1))
    rc, res, _, _ = srv.wait(jid)
    assert rc == _abi.CP_OK and res.status == _abi.CP_ERR_OOM
    srv.check_ok(srv.submit(frames_for(3, seed=2))[1])
    assert_clean(dev, srv.close()[1])


def test_budget_refuses_serialises_and_evicts(dev):
    n, h, w, c = 4, 6, 10, 3
    pitch = (h * w * c + 16 + 255) // 256 * 256
    ob = (h * w * c + 255) // 256 * 256
    job_bytes = n * pitch + 2 * ob + 256
    # a job larger than the whole budget can never run
    srv = Server(dev, budget=job_bytes - 1)
    rc, jid = srv.submit(frames_for(n))
    assert srv.wait(jid)[1].status == _abi.CP_ERR_BUDGET
    assert_clean(dev, srv.close()[1])

    # one job's worth: jobs run one after another, cached frames are evicted for new ones
    dev.mock_reset()
    srv = Server(dev, budget=job_bytes, inflight=4)
    fa, fb = frames_for(n, seed=1), frames_for(n, seed=2)
    ka, kb = [1, 2, 3, 4], [11, 12, 13, 14]
    ids = [srv.submit(fa, ka)[1], srv.submit(fb, kb)[1], srv.submit(fa, ka)[1]]
    res = [srv.check_ok(j) for j in ids]
    for r0, r1 in zip(res, res[1:]):
        assert r1.admit_s >= r0.done_s
    assert frame_uploads(dev) == 3 * n  # every job re-uploads: the budget holds one stack
    assert_clean(dev, srv.close()[1])

    # room for both: keyed frames stay resident and are shared
    dev.mock_reset()
    srv = Server(dev, budget=4 * job_bytes)
    ids = [srv.submit(fa, ka)[1] for _ in range(3)]
    ids.append(srv.submit(fb, [1, 2, 13, 14])[1])  # two frames shared with fa's keys
    fb_shared = fb.copy()
    fb_shared[:2] = fa[:2]
    for jid in ids[:3]:
        srv.check_ok(jid)
    srv.jobs[ids[3]] = (fb_shared,) + srv.jobs[ids[3]][1:]  # what the shared keys mean
    srv.check_ok(ids[3])
    assert frame_uploads(dev) == n + 2
    assert_clean(dev, srv.close()[1])


def test_device_wait_that_gave_up_fails_exactly_its_launch(dev):
    srv = Server(dev, inflight=8)
    dev.mock_hold(HOLD_UPLOADS | HOLD_KERNELS)
    a1, a2 = srv.submit(frames_for(4, seed=1))[1], srv.submit(frames_for(4, seed=2))[1]
    assert poll(lambda: stats(dev)["uploads"] == 8)
    dev.mock_fail_launch_words(1)
    dev.mock_hold(HOLD_KERNELS)  # both uploads land; the jobs go out in one or two launches
    assert poll(lambda: stats(dev)["launches"] >= 1)
    dev.mock_hold(0)
    status = []
    for jid in (a1, a2):
        rc, res, _, _ = srv.wait(jid)
        assert rc == _abi.CP_OK
        status.append(res.status)
    if stats(dev)["max_stacks"] == 2:  # one launch: both jobs read its error word
        assert status == [_abi.CP_ERR_TIMEOUT] * 2
    else:  # the first launch had the word set, the second a clear one
        assert sorted(status) == sorted([_abi.CP_ERR_TIMEOUT, _abi.CP_OK])
    srv.check_ok(srv.submit(frames_for(4, seed=3))[1])  # the next launch has a clear word
    assert_clean(dev, srv.close()[1])


def test_sticky_device_fault_fails_every_job_without_hanging(dev):
    srv = Server(dev, inflight=2)
    dev.mock_fault_launches(1)
    a = srv.submit(frames_for(3, seed=1))[1]
    rc, res, _, _ = srv.wait(a)
    assert rc == _abi.CP_OK and res.status == _abi.CP_ERR_CUDA
    b = srv.submit(frames_for(3, seed=2))[1]
    rc, res, _, _ = srv.wait(b)
    assert rc == _abi.CP_OK and res.status == _abi.CP_ERR_CUDA
    rc, used = srv.close()
    assert used == 0  # the budget is returned even though the device no longer runs frees


def test_launch_slots_are_reused_only_after_their_results_are_read(dev):
    """Nine launch groups against six launch slots: with downloads held no slot frees, so only
    six launches go out; releasing them lets the rest through, every job with its own results.
    A slot reused before its error word was read back would let a later launch's descriptors
    and word overwrite it."""
    srv = Server(dev, inflight=16)
    dev.mock_hold(HOLD_DOWNLOADS)
    ids = []
    for i, (c, n) in enumerate((c, n) for c in (1, 3, 4) for n in (4, 40, 70)):
        ids.append(srv.submit(frames_for(n, c=c, seed=i))[1])
    assert poll(lambda: stats(dev)["launches_run"] == 6)
    time.sleep(0.05)
    assert stats(dev)["launches"] == 6
    dev.mock_hold(0)
    for jid in ids:
        srv.check_ok(jid)
    assert stats(dev)["launches"] == 9
    assert_clean(dev, srv.close()[1])


def test_submit_validates_options_with_the_real_preparation(dev):
    srv = Server(dev)
    assert srv.submit(frames_for(3, c=2))[0] == _abi.CP_ERR_ARG
    assert srv.submit(frames_for(2), thr_abs=0)[0] == _abi.CP_ERR_ARG  # rel needs 3 samples
    assert "relative threshold" in srv.last_error()
    assert srv.submit(frames_for(3), mode=7)[0] == _abi.CP_ERR_ARG
    assert srv.submit(frames_for(3), background=9)[0] == _abi.CP_ERR_ARG
    assert srv.submit(frames_for(_abi.MAX_FRAMES + 1, h=1, w=1))[0] == _abi.CP_ERR_ARG
    assert stats(dev)["uploads"] == 0
    assert_clean(dev, srv.close()[1])


def test_destroy_finishes_queued_and_running_jobs(dev):
    srv = Server(dev, inflight=2)
    bufs = [srv.submit(frames_for(5, seed=i)) for i in range(6)]
    assert all(rc == _abi.CP_OK for rc, _ in bufs)
    kept = dict(srv.jobs)
    rc, used = srv.close()
    assert rc == _abi.CP_OK
    for frames, out, bl, _ in kept.values():
        np.testing.assert_array_equal(out, frames.max(axis=0))
        np.testing.assert_array_equal(bl, frames.min(axis=0))
    assert_clean(dev, used)


def test_concurrent_clients_with_shared_keys_and_a_tight_budget(dev):
    h, w = 6, 10
    pitch = (h * w * 3 + 16 + 255) // 256 * 256
    srv = Server(dev, budget=40 * pitch, inflight=6)
    pool = frames_for(24, h, w, 3, seed=5)
    errors = []

    def client(t):
        rng = np.random.default_rng(100 + t)
        try:
            for _ in range(15):
                n = int(rng.integers(1, 9))
                idx = np.sort(rng.choice(24, n, replace=False))
                rc, jid = srv.submit(pool[idx], keys=[int(i) + 1 for i in idx],
                                     blend=bool(rng.integers(0, 2)))
                assert rc == _abi.CP_OK
                srv.check_ok(jid)
        except Exception as e:  # reported on the main thread
            errors.append(e)

    th = [threading.Thread(target=client, args=(t,)) for t in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join(60)
    assert not errors, errors[0]
    assert frame_uploads(dev) < 4 * 15 * 8  # resident frames were shared
    assert_clean(dev, srv.close()[1])

