"""Per-frame feature cap (uslam_params.frame_cap): the levels fill in order,
each keeping what the earlier levels left of the cap, so a frame keeps the
first frame_cap features in (level, order within the level) order.  The GPU
equals the oracle's statement of that policy, alone and with per-cell caps,
and the brute-force matchers see exactly those features."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, synth

pytestmark = pytest.mark.gpu


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


@pytest.mark.parametrize("frame_cap,cell_cap,matcher", [(3000, 0, 0), (2200, 3, 0), (2500, 0, 2), (5, 0, 1),
                                                         (10 ** 6, 0, 0)])
def test_frame_cap_equals_oracle(brief_pattern, frame_cap, cell_cap, matcher):
    W, H, L = 1280, 720, 8
    frames = list(synth.warped_pair(61, W, H))
    cap = 3000
    exp = [oracle.frame(f, brief_pattern, levels=L, cap=cap, cell_cap=cell_cap, frame_cap=frame_cap) for f in frames]
    with Context(brief_pattern, levels=L, max_width=W, max_height=H, cap_per_level=cap, cell_cap=cell_cap,
                 frame_cap=frame_cap, matcher=matcher, ratio=0.8) as ctx:
        b = Batch(ctx, [(W, H)] * 2, [(0, 1)])
        try:
            b.process(frames)
            for i in range(2):
                gf, gk, gr = b.features(i)
                assert np.array_equal(gr, exp[i][2]) and np.array_equal(gk, exp[i][1]), (i, gk, exp[i][1])
                assert gf.tobytes() == exp[i][0].tobytes(), f"frame {i}"
                assert int(gk.sum()) == min(frame_cap, int(exp[i][1].sum()))
            if matcher == 0:
                em = oracle.match(exp[0][0], exp[0][1], exp[1][0], exp[1][1], W, H)
            else:
                em = oracle.match_bruteforce(exp[0][0], exp[0][1], exp[1][0], exp[1][1], 0.8)
            assert np.array_equal(_mm(b.matches(0)), em)
        finally:
            b.close()
