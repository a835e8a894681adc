"""k_match keeps one b -> a accumulator per (pair, current feature): pairs that
share a current frame, or use a frame as previous in one pair and current in
another, must each equal the oracle.  A batch whose (pair, level) segments
exceed what one k_match launch takes is refused at creation."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, synth
from uni_slam_gb300.capi import USlamError

pytestmark = pytest.mark.gpu

W, H = 320, 240


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def test_pairs_sharing_a_current_frame(brief_pattern):
    f0, f1 = synth.warped_pair(41, W, H)
    f2 = synth.warped_pair(42, W, H)[1]
    frames = [f0, f1, f2]
    # frame 2 is current in two pairs; frame 0 is previous in one and current in another
    pairs = [(0, 2), (1, 2), (2, 0), (1, 0)]
    exp = [oracle.frame(f, brief_pattern) for f in frames]
    with Context(brief_pattern, levels=6, max_width=W, max_height=H) as ctx:
        b = Batch(ctx, [(W, H)] * 3, pairs)
        try:
            b.process(frames)
            got = [_mm(b.matches(p)) for p in range(len(pairs))]
        finally:
            b.close()
    for p, (a, c) in enumerate(pairs):
        em = oracle.match(exp[a][0], exp[a][1], exp[c][0], exp[c][1], W, H)
        assert np.array_equal(got[p], em), f"pair {p} {pairs[p]}"
    assert sum(len(g) for g in got) > 0


def test_match_segment_limit(brief_pattern):
    # 342 pairs x 6 levels = 2052 (pair, level) segments, over the 2048 one
    # k_match launch takes
    n = 343
    with Context(brief_pattern, levels=6, max_width=64, max_height=64) as ctx:
        with pytest.raises(USlamError) as e:
            Batch(ctx, [(64, 64)] * n, [(i, i + 1) for i in range(n - 1)])
        assert "2048" in str(e.value)
        b = Batch(ctx, [(64, 64)] * (n - 1), [(i, i + 1) for i in range(n - 2)])  # 2046 segments
        b.close()
