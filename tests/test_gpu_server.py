"""The continuous-batching server (needs a GB300): every job's result is the same alone and
in the mix; keyed frames are shared between jobs; the HBM budget is enforced."""
import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import _abi
from oracle import oracle
from tests import cases

pytestmark = pytest.mark.gpu

MODES = [dict(outlier="extreme", background="first"), dict(outlier="average", background="average"),
         dict(outlier="first", background="median"), dict(outlier="last", background="random"),
         dict(outlier="forward", background="first", threshold="rel/2/4")]


def test_results_same_alone_and_in_mix(ctx):
    rng = np.random.default_rng(0)
    jobs = []
    for i in range(14):
        n = int(rng.integers(3, 70))
        h, w = [(16, 24), (40, 64), (33, 70), (64, 64)][i % 4]
        c = 1 if i % 5 == 4 else 3
        frames = cases.random_stack(rng, n, h, w, c, n_spots=4)
        kw = dict(MODES[i % len(MODES)])
        if i % 7 == 6:
            kw = dict(mode="lighter")
        jobs.append((frames, kw))
    alone = [ctx.composite(f, cases.params(**kw)) for f, kw in jobs]
    with cg.Server(ctx, max_inflight=6) as srv:
        ids = [srv.submit(f, cases.params(**kw)) for f, kw in jobs]
        res = [srv.wait(j) for j in ids]
    for (f, kw), a, r in zip(jobs, alone, res):
        assert r["status"] == 0
        assert np.array_equal(r["out"], a[0])
        if kw.get("mode", "outlier") == "outlier":
            assert np.array_equal(r["blend"], a[1])
            assert r["warnings"] == a[2]
        assert r["submit_s"] <= r["admit_s"] <= r["done_s"]


def test_many_launches_all_succeed(ctx):
    """Hundreds of jobs in bursts, so that launch slots are reused while the results of their
    previous launches are still being read back, with batches of varying size (descriptor
    arrays of varying length in the reused slot memory): every job succeeds with the result
    of its lone composite."""
    rng = np.random.default_rng(5)
    base = [cases.random_stack(rng, 40, 120, 160, 3, n_spots=4) for _ in range(4)]
    specs = []
    for i in range(240):
        n = int(rng.integers(3, 40))
        specs.append((i % 4, n, MODES[i % 4]))
    alone = {}
    for b, n, kw in specs:
        if (b, n, kw["outlier"]) not in alone:
            alone[(b, n, kw["outlier"])] = ctx.composite(base[b][:n], cases.params(**kw))[0]
    with cg.Server(ctx, max_inflight=8) as srv:
        ids, done = [], {}
        for k in range(0, len(specs), 24):
            ids += [srv.submit(base[b][:n], cases.params(**kw)) for b, n, kw in specs[k:k + 24]]
            done[ids[-1]] = srv.wait(ids[-1])  # the burst's last job: the others mostly done
        res = [done[j] if j in done else srv.wait(j) for j in ids]
    assert [r["status"] for r in res] == [0] * len(specs)
    for (b, n, kw), r in zip(specs, res):
        assert np.array_equal(r["out"], alone[(b, n, kw["outlier"])])


def test_shared_keyed_frames(ctx):
    """Overlapping windows submitted with frame keys: frames upload once and are shared."""
    rng = np.random.default_rng(1)
    pool = cases.random_stack(rng, 20, 24, 40, 3, n_spots=5)
    wins = [list(range(s, s + 8)) for s in range(0, 13)]
    with cg.Server(ctx) as srv:
        ids = [srv.submit(pool[w], cases.params(outlier="forward", background="first",
                                                fade="clamp/abs/0,0.5/12,1"),
                          keys=[1000 + i for i in w], frame_offset=w[0]) for w in wins]
        res = [srv.wait(j) for j in ids]
    for w, r in zip(wins, res):
        p = cases.params(outlier="forward", background="first", fade="clamp/abs/0,0.5/12,1")
        ref = oracle.composite(pool[w], p, frame_offset=w[0])
        assert r["status"] == 0
        assert np.array_equal(r["out"], ref[0]) and np.array_equal(r["blend"], ref[1])


def test_budget(ctx):
    rng = np.random.default_rng(2)
    small = cases.random_stack(rng, 4, 16, 16, 3)
    big = cases.random_stack(rng, 40, 128, 128, 3)  # ~2 MB of frames
    with cg.Server(ctx, hbm_budget=1 << 20) as srv:
        a = srv.submit(small, cases.params())
        b = srv.submit(big, cases.params())
        ra, rb = srv.wait(a), srv.wait(b)
    assert ra["status"] == 0 and rb["status"] == _abi.CP_ERR_BUDGET


def test_invalid_job_rejected(ctx):
    with cg.Server(ctx) as srv:
        with pytest.raises(_abi.ChronoError):
            srv.submit(np.zeros((2, 4, 4, 3), np.uint8), cases.params(threshold="rel/1/2"))


def test_cancel_queued_jobs(ctx):
    """With one job in flight at a time, jobs still in the queue can be cancelled: they
    complete with CP_ERR_CANCELLED and the others are unaffected."""
    rng = np.random.default_rng(12)
    frames = [cases.random_stack(rng, 40, 64, 96, 3, n_spots=4) for _ in range(8)]
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                     background="first")
    with cg.Server(ctx, max_inflight=1) as srv:
        ids = [srv.submit(f, p) for f in frames]
        cancelled = [srv.cancel(i) for i in ids[4:]]
        res = [srv.wait(i) for i in ids]
    assert any(cancelled)
    for f, r, c in zip(frames, res, [False] * 4 + cancelled):
        if c:
            assert r["status"] == _abi.CP_ERR_CANCELLED
        else:
            assert r["status"] == 0
            ref = oracle.composite(f, p)
            cases.assert_close_u8(r["out"], ref[0], what="served composite")


def test_server_reports_timeouts_and_allocation_failures(ctx):
    """A launch whose bounded waits give up fails exactly its jobs with CP_ERR_TIMEOUT; an
    injected allocation failure fails the job being admitted with CP_ERR_OOM; jobs after
    either run normally on the same server."""
    rng = np.random.default_rng(13)
    frames = cases.random_stack(rng, 20, 48, 64, 3, n_spots=3)
    p = cases.params(mode="outlier", threshold="abs/0.05/0.2", outlier="average",
                     background="first")
    ref = oracle.composite(frames, p)
    lib = _abi.lib()
    with cg.Server(ctx, max_inflight=2) as srv:
        assert lib.cp_ctx_set_wait_limit(ctx.handle, 1) == 0
        try:
            r = srv.wait(srv.submit(frames, p))
        finally:
            assert lib.cp_ctx_set_wait_limit(ctx.handle, 0) == 0
        assert r["status"] == _abi.CP_ERR_TIMEOUT
        assert lib.cp_ctx_fail_allocations(ctx.handle, 1) == 0
        try:
            r = srv.wait(srv.submit(frames, p))
        finally:
            assert lib.cp_ctx_fail_allocations(ctx.handle, 0) == 0
        assert r["status"] == _abi.CP_ERR_OOM
        r = srv.wait(srv.submit(frames, p))
        assert r["status"] == 0
        cases.assert_close_u8(r["out"], ref[0], what="after failures")
