"""Per-32x32-cell caps in the oracle against a numpy statement of the policy:
cells of each level in row-major order, (y, x) order inside a cell, the
first cell_cap keypoints of every cell, then the level cap over that list;
raw counts are the pre-cap keypoint counts."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import synth


def _culled_levels(img, levels):
    H0, W0 = img.shape
    out = []
    for l in range(levels):
        lvl = oracle.pyramid_level(img, l, levels)
        out.append(oracle.cull(oracle.detect(lvl), W0, H0))
    return out


def _expected(culled, cap, cell_cap):
    h, w = culled.shape
    pts = []
    for cy in range(0, h, 32):
        for cx in range(0, w, 32):
            ys, xs = np.nonzero(culled[cy:cy + 32, cx:cx + 32])
            order = np.lexsort((xs, ys))[:cell_cap]
            pts += [(cx + xs[i], cy + ys[i]) for i in order]
    return pts[:cap]


@pytest.mark.parametrize("size,cap,cell_cap", [((640, 480), 1228, 3), ((203, 97), 30, 1), ((752, 480), 400, 8)])
def test_cell_caps_follow_policy(brief_pattern, size, cap, cell_cap):
    w, h = size
    img = synth.scene_frame(17, w, h)
    feats, kept, raw = oracle.frame(img, brief_pattern, levels=6, cap=cap, cell_cap=cell_cap)
    culled = _culled_levels(img, 6)
    off = 0
    for l, c in enumerate(culled):
        exp = _expected(c, cap, cell_cap)
        assert raw[l] == np.count_nonzero(c)
        assert kept[l] == len(exp)
        got = feats[off:off + kept[l]]
        assert [(int(f["x"]), int(f["y"])) for f in got] == exp
        assert all(int(f["strength"]) == int(c[y, x]) for f, (x, y) in zip(got, exp))
        off += kept[l]
    assert off == len(feats)


def test_cell_cap_zero_is_the_yx_policy(brief_pattern):
    img = synth.scene_frame(4)
    a = oracle.frame(img, brief_pattern, cell_cap=0)
    b = oracle.frame(img, brief_pattern)
    assert a[0].tobytes() == b[0].tobytes() and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("frame_cap,cell_cap", [(3000, 0), (1500, 2), (10, 0), (100000, 0)])
def test_frame_cap_keeps_the_first_in_level_order(brief_pattern, frame_cap, cell_cap):
    """The per-frame cap keeps the first frame_cap features of the uncapped
    frame in (level, order within the level) order: the levels fill in order."""
    img = synth.scene_frame(9, 752, 480)
    full, fk, fr = oracle.frame(img, brief_pattern, cell_cap=cell_cap)
    got, gk, gr = oracle.frame(img, brief_pattern, cell_cap=cell_cap, frame_cap=frame_cap)
    assert np.array_equal(gr, fr)
    n = min(frame_cap, int(fk.sum()))
    assert int(gk.sum()) == n and got.tobytes() == full[:n].tobytes()
    left = frame_cap
    for l in range(len(fk)):
        assert gk[l] == min(fk[l], max(left, 0))
        left -= gk[l]
