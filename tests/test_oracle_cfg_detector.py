"""The oracle's cfg detection profile (FAST 9-of-16 with wrap-around at
20/255, sum-of-excess score, 3x3 NMS with ties to the first pixel in raster
order, 3-pixel border excluded) against a vectorised numpy statement of the
same definition, plus a hand-checked corner and the frame-level wiring."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import synth

CX = [0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3, -3, -3, -2, -1]
CY = [-3, -3, -2, -1, 0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3]
T = np.float32(20.0) / np.float32(255.0)


def _circ_run(m):
    m = m.astype(np.uint64)
    x = (m | (m << np.uint64(16))) & np.uint64(0xFFFFFFFF)
    run = np.zeros(m.shape, np.int64)
    while np.any(x):
        nz = x != 0
        run += nz
        x = x & ((x << np.uint64(1)) & np.uint64(0xFFFFFFFF))
    return np.where(m == 0xFFFF, 16, run)


def _numpy_cfg(lvl):
    h, w = lvl.shape
    c = lvl[3:h - 3, 3:w - 3]
    pts = [lvl[3 + dy:h - 3 + dy, 3 + dx:w - 3 + dx] for dx, dy in zip(CX, CY)]
    mb = sum(((p - c) > T).astype(np.int64) << i for i, p in enumerate(pts))
    md = sum(((c - p) > T).astype(np.int64) << i for i, p in enumerate(pts))
    rb, rd = _circ_run(mb), _circ_run(md)
    bright = rb >= 9
    corner = (rb >= 9) | (rd >= 9)
    m = np.where(bright, mb, md)
    sc = np.zeros(c.shape, np.float32)
    for i, p in enumerate(pts):
        term = np.where(bright, (p - c), (c - p)) - T
        sc = np.where(((m >> i) & 1).astype(bool), (sc + term).astype(np.float32), sc)
    score = np.zeros((h, w), np.float32)
    arc = np.zeros((h, w), np.int64)
    score[3:h - 3, 3:w - 3] = np.where(corner, sc, 0)
    arc[3:h - 3, 3:w - 3] = np.where(corner, np.where(bright, rb, rd), 0)
    pad = np.pad(score, 1)
    keep = arc > 0
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            if dy == 0 and dx == 0:
                continue
            q = pad[1 + dy:1 + dy + h, 1 + dx:1 + dx + w]
            earlier = dy < 0 or (dy == 0 and dx < 0)
            keep &= (score > q) if earlier else (score >= q)
    return np.where(keep, arc, 0).astype(np.uint32)


@pytest.mark.parametrize("seed,size,level", [(1, (160, 120), 0), (2, (203, 97), 1), (3, (320, 240), 2)])
def test_cfg_detector_matches_numpy(seed, size, level):
    img = synth.scene_frame(seed, *size)
    lvl = oracle.pyramid_level(img, level)
    got = oracle.detect_cfg(lvl)
    exp = _numpy_cfg(lvl)
    assert np.array_equal(got, exp)
    assert np.count_nonzero(got) > 5


def test_cfg_square_corner_and_plateau_tie():
    lvl = np.zeros((40, 40), np.float32)
    lvl[10:30, 10:30] = np.float32(200) / np.float32(255)
    got = oracle.detect_cfg(lvl)
    ys, xs = np.nonzero(got)
    pts = set(zip(xs.tolist(), ys.tolist()))
    # each convex corner of the bright square yields one surviving corner next to it
    for cx, cy in [(10, 10), (29, 10), (10, 29), (29, 29)]:
        assert any(abs(x - cx) <= 1 and abs(y - cy) <= 1 for x, y in pts), (cx, cy, pts)
    assert all(9 <= got[y, x] <= 16 for x, y in pts)
    # flat image: nothing; the 3-pixel border never fires
    assert not oracle.detect_cfg(np.full((20, 20), 0.5, np.float32)).any()


def test_cfg_frame_uses_cfg_detector(brief_pattern):
    img = synth.scene_frame(6)
    feats, kept, raw = oracle.frame(img, brief_pattern, detector=1)
    lvl0 = oracle.pyramid_level(img, 0)
    m = oracle.detect_cfg(lvl0)
    assert raw[0] == np.count_nonzero(m)
    ys, xs = np.nonzero(m)
    k0 = feats[:kept[0]]
    assert np.array_equal(k0["x"].astype(int), xs[:kept[0]]) and np.array_equal(k0["y"].astype(int), ys[:kept[0]])
    assert np.array_equal(k0["strength"], m[ys[:kept[0]], xs[:kept[0]]])
