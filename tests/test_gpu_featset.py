"""The single-frame export set through the C ABI: uslam_detect_describe (u8)
and uslam_detect_describe_f32 (the reference's f32 u8/255 frames) into
device-resident feature sets, their host copies, and uslam_match_sets between
two sets, against the oracle; frame-size mismatches are refused."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Context, FeatureSet, USlamError, synth

pytestmark = pytest.mark.gpu


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def test_detect_describe_and_match_sets(brief_pattern):
    f0, f1 = synth.warped_pair(21)
    e0, e1 = oracle.frame(f0, brief_pattern), oracle.frame(f1, brief_pattern)
    with Context(brief_pattern, levels=6, max_width=752, max_height=480) as c:
        with FeatureSet(c, 752, 480) as a, FeatureSet(c, 752, 480) as b:
            a.detect(f0)
            b.detect((f1.astype(np.float32) / np.float32(255.0)).astype(np.float32))  # f32 FrameBW input
            for fs, e in ((a, e0), (b, e1)):
                gf, gk, gr = fs.features()
                assert np.array_equal(gk, e[1]) and np.array_equal(gr, e[2])
                assert gf.tobytes() == e[0].tobytes()
            em = oracle.match(e0[0], e0[1], e1[0], e1[1], 752, 480)
            assert np.array_equal(_mm(c.match(a, b)), em) and len(em) > 500
            # the same sets again, and reversed
            assert np.array_equal(_mm(c.match(a, b)), em)
            er = oracle.match(e1[0], e1[1], e0[0], e0[1], 752, 480)
            assert np.array_equal(_mm(c.match(b, a)), er)
            with FeatureSet(c, 640, 480) as other:
                other.detect(synth.scene_frame(5, 640, 480))
                with pytest.raises(USlamError):
                    c.match(a, other)
                with pytest.raises(USlamError):
                    other.detect(f0)  # 752x480 frame into a 640x480 set


def test_match_sets_bruteforce(brief_pattern):
    f0, f1 = synth.warped_pair(22, 640, 480)
    e0, e1 = oracle.frame(f0, brief_pattern), oracle.frame(f1, brief_pattern)
    with Context(brief_pattern, levels=6, max_width=640, max_height=480, matcher=1, ratio=0.8) as c:
        with FeatureSet(c, 640, 480) as a, FeatureSet(c, 640, 480) as b:
            a.detect(f0)
            b.detect(f1)
            em = oracle.match_bruteforce(e0[0], e0[1], e1[0], e1[1], 0.8)
            assert np.array_equal(_mm(c.match(a, b)), em) and len(em) > 200


def test_last_error_from_many_threads(brief_pattern):
    """Calls failing on one context from several host threads at once (the
    served form's submitting threads can do this): every thread's
    uslam_last_error reads a whole message.  The failing call, features of a
    set with nothing detected, does no GPU work."""
    import threading

    from uni_slam_gb300 import capi

    with Context(brief_pattern, levels=6, max_width=64, max_height=64) as c:
        lib = c.lib
        sets = [FeatureSet(c, 64, 64) for _ in range(4)]
        statuses, msgs = [], []

        def worker(fs):
            kept = np.zeros(6, np.int32)
            raw = np.zeros(6, np.int32)
            for _ in range(2000):
                statuses.append(lib.uslam_featset_features(fs.h, None, 0, capi.iptr(kept), capi.iptr(raw)))
                msgs.append(lib.uslam_last_error(c.h))

        threads = [threading.Thread(target=worker, args=(fs,)) for fs in sets]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for fs in sets:
            fs.close()
        assert set(statuses) == {capi.NOT_READY}
        assert set(msgs) == {b"featset_features: nothing detected yet"}
