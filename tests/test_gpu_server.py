"""Served form: each stream's results are the same alone and in a mix of
concurrent streams (continuous batching), equal the oracle (features, and
matches against the stream's keyframe), and admission refuses a frame when
the HBM budget has no free slot."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Context, Server, synth

pytestmark = pytest.mark.gpu

SIZES = [(640, 480), (752, 480), (1280, 720)]


def _rows(m):
    if m is None or len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def _run_streams(ctx, streams, promote_every=3, budget=2 << 30):
    """streams: list of frame lists.  Submits round-robin without waiting
    (frames of several streams queue together) and returns per-stream results."""
    srv = Server(ctx, SIZES, hbm_budget_bytes=budget, max_batch=64)
    try:
        ids = [srv.open_stream(f[0].shape[1], f[0].shape[0]) for f in streams]
        tickets = [[] for _ in streams]
        n = max(len(f) for f in streams)
        for i in range(n):
            for s, frames in enumerate(streams):
                if i < len(frames):
                    t = srv.submit(ids[s], frames[i], promote=(i % promote_every == 0))
                    assert t is not None
                    tickets[s].append(t)
        out = []
        for s in range(len(streams)):
            res = []
            for t in tickets[s]:
                srv.wait(t, 60000)
                f, kept, raw, m, _ = srv.result(t)
                res.append((f.tobytes(), kept.copy(), raw.copy(), _rows(m)))
                srv.release(t)
            out.append(res)
        stats = srv.stats()
        return out, stats
    finally:
        srv.close()


def test_alone_equals_in_mix_and_oracle(brief_pattern):
    ctx = Context(brief_pattern, levels=6, max_width=1280, max_height=720)
    try:
        mine = synth.plane_sequence(31, n=5)
        others = [synth.plane_sequence(40 + k, n=5, w=SIZES[k % 3][0], h=SIZES[k % 3][1]) for k in range(5)]
        alone, _ = _run_streams(ctx, [mine])
        mixed, stats = _run_streams(ctx, others[:2] + [mine] + others[2:])
        assert stats["max_batch_seen"] > 1  # frames of several streams shared launches
        for a, b in zip(alone[0], mixed[2]):
            assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[3], b[3])
        # oracle: features, and matches against the keyframe (frames 0 and 3 promote)
        exp = [oracle.frame(f, brief_pattern) for f in mine]
        for i, (fb, kept, raw, m) in enumerate(alone[0]):
            assert fb == exp[i][0].tobytes() and np.array_equal(kept, exp[i][1]) and np.array_equal(raw, exp[i][2])
            if i == 0:
                assert len(m) == 0
                continue
            key = 0 if i <= 3 else 3
            em = oracle.match(exp[key][0], exp[key][1], exp[i][0], exp[i][1], 752, 480)
            assert np.array_equal(m, em), f"frame {i}"
    finally:
        ctx.close()


def test_admission_refuses_without_a_free_slot(brief_pattern):
    ctx = Context(brief_pattern, levels=6, max_width=752, max_height=480)
    try:
        frames = synth.plane_sequence(3, n=4)
        # a budget of 2 slots per size class (about 10 MB per 752x480 slot)
        srv = Server(ctx, [(752, 480)], hbm_budget_bytes=22 << 20, max_batch=8)
        try:
            assert srv.stats()["slots"] == 2
            sid = srv.open_stream(752, 480)
            t0 = srv.submit(sid, frames[0])       # keyframe: slot 1 of 2
            t1 = srv.submit(sid, frames[1])       # slot 2 of 2
            assert t0 is not None and t1 is not None
            assert srv.submit(sid, frames[2]) is None  # no free slot: refused
            srv.wait(t1, 60000)
            srv.release(t1)
            t2 = srv.submit(sid, frames[2])       # the released slot is reused
            assert t2 is not None
            srv.wait(t2, 60000)
            assert srv.result(t2)[3] is not None
            srv.wait(t0, 60000)
            srv.release(t0)
            srv.release(t2)
        finally:
            srv.close()
    finally:
        ctx.close()


def test_failure_finishes_queued_requests(brief_pattern):
    """The served form's failure path, without any GPU fault: with 0 polls for
    the first wait of k_detect's tile load, every launch trips its kernel check
    (USLAM_ERR_TMA_TIMEOUT, recorded once the copy in flight has landed).  With
    one frame per launch, at most two launches are in flight and the rest of
    the frames queue; the launches in flight and the queued requests all
    finish with USLAM_KERNEL_CHECK (bounded waits: a request left unfinished
    would time out instead), and the server refuses new frames with it."""
    from uni_slam_gb300 import USlamError, capi

    ctx = Context(brief_pattern, levels=6, max_width=752, max_height=480)
    try:
        frames = synth.plane_sequence(9, n=8)
        srv = Server(ctx, [(752, 480)], hbm_budget_bytes=256 << 20, max_batch=1)
        try:
            sid = srv.open_stream(752, 480)
            ctx.check(ctx.lib.uslam_server_set_first_wait(srv.h, 0), "set_first_wait")
            tickets = []
            for f in frames:
                try:
                    t = srv.submit(sid, f)
                except USlamError as e:  # the first launch already failed
                    assert e.status == capi.KERNEL_CHECK
                    break
                assert t is not None
                tickets.append(t)
            assert tickets
            for t in tickets:
                with pytest.raises(USlamError) as ei:
                    srv.wait(t, 10000)
                assert ei.value.status == capi.KERNEL_CHECK, str(ei.value)
                # no results for a failed request
                with pytest.raises(USlamError) as ei:
                    srv.result(t)
                assert ei.value.status == capi.KERNEL_CHECK, str(ei.value)
                srv.release(t)
            with pytest.raises(USlamError) as ei:
                srv.submit(sid, frames[0])
            assert ei.value.status == capi.KERNEL_CHECK
        finally:
            srv.close()
    finally:
        ctx.close()
