"""Batched-uneven form: every detect tile shape (alone and mixed in one
batch) is bit-exact with the oracle, the autotuner stores its choice per
resolution class without changing any result, and per-32x32-cell caps match
the oracle's cell policy on an uneven batch with each frame matched against a
seeded warp of itself."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, synth

pytestmark = pytest.mark.gpu

SIZES = [(640, 480), (752, 480), (1280, 720), (1920, 1080), (203, 97)]


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def _check_features(b, frames, exp):
    for i in range(len(frames)):
        gf, gk, gr = b.features(i)
        assert np.array_equal(gr, exp[i][2]) and np.array_equal(gk, exp[i][1]), f"frame {i}"
        assert gf.tobytes() == exp[i][0].tobytes(), f"frame {i}"


def test_every_tile_shape_bit_exact(brief_pattern):
    frames = [synth.scene_frame(50 + i, w, h) for i, (w, h) in enumerate(SIZES)]
    exp = [oracle.frame(f, brief_pattern) for f in frames]
    with Context(brief_pattern, levels=6, max_width=1920, max_height=1080) as c:
        n = len(c.tile_shapes())
        assert n >= 2
        for s in range(n):
            for w, h in SIZES:
                c.set_tile_shape(w, h, s)
            b = Batch(c, SIZES, [])
            try:
                b.process(frames)
                _check_features(b, frames, exp)
            finally:
                b.close()
        # several shapes in one batch (one detect launch per shape)
        for k, (w, h) in enumerate(SIZES):
            c.set_tile_shape(w, h, k % n)
        b = Batch(c, SIZES, [])
        try:
            b.process(frames)
            _check_features(b, frames, exp)
        finally:
            b.close()


def test_autotune_stores_choice_and_keeps_results(brief_pattern):
    f0, f1 = synth.warped_pair(8, 1280, 720)
    with Context(brief_pattern, levels=6, max_width=1280, max_height=720) as c:
        shape, ms = c.autotune(f0, n_frames=4, reps=3)
        assert 0 <= shape < len(c.tile_shapes())
        assert all(m > 0 for m in ms) and ms[shape] == min(ms)
        assert c.tile_shape(1280, 720) == shape
        assert c.tile_shape(640, 480) == 0  # untouched classes keep the default
        b = Batch(c, [(1280, 720), (1280, 720)], [(0, 1)])
        try:
            b.process([f0, f1])
            ea, eb = oracle.frame(f0, brief_pattern), oracle.frame(f1, brief_pattern)
            _check_features(b, [f0, f1], [ea, eb])
            em = oracle.match(ea[0], ea[1], eb[0], eb[1], 1280, 720)
            assert np.array_equal(_mm(b.matches(0)), em) and len(em) > 100
        finally:
            b.close()


def test_cell_caps_uneven_batch(brief_pattern):
    sizes = [(640, 480), (1280, 720), (203, 97), (752, 480)]
    frames, pairs = [], []
    for k, (w, h) in enumerate(sizes):
        a, b = synth.warped_pair(70 + k, w, h)
        pairs.append((len(frames), len(frames) + 1))
        frames += [a, b]
    with Context(brief_pattern, levels=6, max_width=1280, max_height=720, cell_cap=4) as c:
        c.set_tile_shape(1280, 720, 1)
        b = Batch(c, [(f.shape[1], f.shape[0]) for f in frames], pairs)
        try:
            b.process(frames)
            exp = [oracle.frame(f, brief_pattern, cell_cap=4) for f in frames]
            _check_features(b, frames, exp)
            plain = oracle.frame(frames[0], brief_pattern)
            assert exp[0][1].sum() < plain[1].sum()  # the cell caps bind
            for k, (p, q) in enumerate(pairs):
                W0, H0 = sizes[k]
                em = oracle.match(exp[p][0], exp[p][1], exp[q][0], exp[q][1], W0, H0)
                assert np.array_equal(_mm(b.matches(k)), em), f"pair {k}"
        finally:
            b.close()
