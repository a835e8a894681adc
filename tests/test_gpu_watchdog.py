"""Host-side watchdog, exercised without any GPU fault: a bounded wait on
queued work returns USLAM_TIMEOUT and leaves the batch usable, and the work
then completes with results equal to the oracle."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, USlamError, capi, synth

pytestmark = pytest.mark.gpu


def test_batch_sync_timeout_then_completes(brief_pattern):
    frames = synth.plane_sequence(5, n=16)
    with Context(brief_pattern, levels=6, max_width=752, max_height=480) as c:
        b = Batch(c, [(752, 480)] * 16, [(i, i + 1) for i in range(15)])
        try:
            for i, f in enumerate(frames):
                b.set_frame(i, f)
            b.upload()
            for _ in range(200):  # ~0.15 s of queued graph replays
                b.run()
            b.download()
            with pytest.raises(USlamError) as ei:
                b.sync(timeout_ms=1)
            assert ei.value.status == capi.TIMEOUT
            b.sync()  # no limit: the queued work finishes
            gf, gk, gr = b.features(7)
            e = oracle.frame(frames[7], brief_pattern)
            assert gf.tobytes() == e[0].tobytes() and np.array_equal(gk, e[1])
        finally:
            b.close()


def _mm(m):
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1) if len(m) else np.zeros((0, 4), np.int32)


@pytest.mark.parametrize("matcher,detect_polls,match_polls", [(0, 0, -1), (2, -1, 0)])
def test_first_wait_runs_out_then_clean_run(brief_pattern, matcher, detect_polls, match_polls):
    """The kernels' bounded device waits, made to run out without any fault:
    with 0 polls for the first wait of k_detect's tile load (or of the
    tensor-core matcher's first query-tile load), the kernel records
    USLAM_ERR_TMA_TIMEOUT once the copy in flight has landed, the batch
    reports USLAM_KERNEL_CHECK, and with the limit restored the next run is
    clean and equals the oracle."""
    W, H = 320, 240
    f1, f2 = synth.warped_pair(41, W, H)
    with Context(brief_pattern, levels=6, max_width=W, max_height=H, matcher=matcher, ratio=0.8) as c:
        b = Batch(c, [(W, H)] * 2, [(0, 1)])
        try:
            for i, f in enumerate((f1, f2)):
                b.set_frame(i, f)
            b.upload()
            c.check(c.lib.uslam_batch_set_first_wait(b.h, detect_polls, match_polls), "set_first_wait")
            b.run()
            with pytest.raises(USlamError) as ei:
                b.sync()
            assert ei.value.status == capi.KERNEL_CHECK
            assert "wait limit" in str(ei.value)
            c.check(c.lib.uslam_batch_set_first_wait(b.h, -1, -1), "set_first_wait")
            b.process([f1, f2])
            exp = [oracle.frame(f, brief_pattern) for f in (f1, f2)]
            for i in range(2):
                gf, gk, _ = b.features(i)
                assert gf.tobytes() == exp[i][0].tobytes() and np.array_equal(gk, exp[i][1])
            if matcher == 0:
                em = oracle.match(exp[0][0], exp[0][1], exp[1][0], exp[1][1], W, H)
            else:
                em = oracle.match_bruteforce(exp[0][0], exp[0][1], exp[1][0], exp[1][1], 0.8)
            assert np.array_equal(_mm(b.matches(0)), em)
        finally:
            b.close()
