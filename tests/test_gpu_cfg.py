"""The cfg profile end to end on the GPU (FAST 9-of-16 at 20/255 with 3x3
NMS, brute-force top-2 matching at ratio 0.8): features bit-exact with the
oracle in every detect tile shape, on uneven sizes down to levels narrower
than the FAST circle, and the brute-force match lists of frame/warp pairs."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, synth

pytestmark = pytest.mark.gpu


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def test_cfg_profile_bit_exact(brief_pattern):
    sizes = [(752, 480), (640, 480), (203, 97), (40, 30)]
    frames, pairs = [], []
    for k, (w, h) in enumerate(sizes):
        a, b = synth.warped_pair(90 + k, w, h)
        pairs.append((len(frames), len(frames) + 1))
        frames += [a, b]
    exp = [oracle.frame(f, brief_pattern, detector=1) for f in frames]
    assert exp[0][2].sum() > 500
    with Context(brief_pattern, levels=6, max_width=752, max_height=480, detector=1, matcher=1, ratio=0.8) as c:
        for shape in range(len(c.tile_shapes())):
            for w, h in sizes:
                c.set_tile_shape(w, h, shape)
            b = Batch(c, [(f.shape[1], f.shape[0]) for f in frames], pairs)
            try:
                b.process(frames)
                for i in range(len(frames)):
                    gf, gk, gr = b.features(i)
                    assert np.array_equal(gr, exp[i][2]) and np.array_equal(gk, exp[i][1]), (shape, i)
                    assert gf.tobytes() == exp[i][0].tobytes(), (shape, i)
                for k, (p, q) in enumerate(pairs):
                    em = oracle.match_bruteforce(exp[p][0], exp[p][1], exp[q][0], exp[q][1], 0.8)
                    assert np.array_equal(_mm(b.matches(k)), em), (shape, k)
                assert len(_mm(b.matches(0))) > 100
            finally:
                b.close()
