"""Batched RANSAC scoring on the GPU (uslam_ransac_score) against the
oracle: inlier counts and bitmasks of many fundamental matrices over the
correspondences of a synthetic two view geometry and of a real matched frame
pair, including ragged and empty match counts."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Context, synth

from test_oracle_ransac import two_view

pytestmark = pytest.mark.gpu


def _hypotheses(rs, p, q, h):
    """Fundamental matrices fitted (numpy 8-point, unnormalised) to random 8-samples."""
    out = []
    for _ in range(h):
        s = rs.choice(len(p), 8, replace=False)
        A = np.c_[q[s, 0:1] * p[s], q[s, 0:1], q[s, 1:2] * p[s], q[s, 1:2], p[s], np.ones((8, 1))]
        out.append(np.linalg.svd(A)[2][-1].reshape(3, 3))
    return np.array(out)


def test_ransac_score_equals_oracle(brief_pattern):
    rs = np.random.RandomState(9)
    F, p, q = two_view(rs, n=1715, outliers=400)
    Fs = np.concatenate([F[None], _hypotheses(rs, p, q, 300), rs.normal(size=(20, 3, 3)), np.zeros((1, 3, 3))])
    with Context(brief_pattern, levels=6, max_width=752, max_height=480) as c:
        for n in (1715, 1000, 33, 1, 0):
            counts, masks = c.ransac_score(Fs, p[:n], q[:n], 3.84, masks=True)
            ec, em = oracle.sampson_counts(Fs, p[:n], q[:n], 3.84)
            assert np.array_equal(counts, ec), n
            assert np.array_equal(masks, em), n
        assert counts.size == len(Fs)
        full = c.ransac_score(Fs, p, q)
        assert full[0] >= 1315 and full[-1] == 0


def test_ransac_score_on_matched_frames(brief_pattern):
    f0, f1 = synth.warped_pair(31)
    a, b = oracle.frame(f0, brief_pattern), oracle.frame(f1, brief_pattern)
    m = oracle.match(a[0], a[1], b[0], b[1], 752, 480)
    aoff = np.concatenate([[0], np.cumsum(a[1])])
    boff = np.concatenate([[0], np.cumsum(b[1])])
    scale = lambda l: np.prod([1.2] * int(l)) if l else 1.0
    p = np.array([[a[0][aoff[la] + ia]["x"] * scale(la), a[0][aoff[la] + ia]["y"] * scale(la)] for la, ia, _, _ in m])
    q = np.array([[b[0][boff[lb] + ib]["x"] * scale(lb), b[0][boff[lb] + ib]["y"] * scale(lb)] for _, _, lb, ib in m])
    Fs = _hypotheses(np.random.RandomState(2), p, q, 500)
    with Context(brief_pattern, levels=6, max_width=752, max_height=480) as c:
        counts = c.ransac_score(Fs, p, q)
    ec, _ = oracle.sampson_counts(Fs, p, q, 3.84)
    assert np.array_equal(counts, ec)
    assert counts.max() > len(m) // 4
