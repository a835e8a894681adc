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
