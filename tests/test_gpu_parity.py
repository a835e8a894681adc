"""Parity of the CUDA path (through the C ABI) with the CPU oracle: bit-exact
pyramid levels, blur cache, culled keypoint maps, feature records
(coordinates, strength, orientation, 256-bit descriptors), raw/kept counts
and mutual match lists, on seeded synthetic frames and edge cases."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, Frontend, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(brief_pattern):
    c = Context(brief_pattern, levels=6, max_width=1280, max_height=720)
    yield c
    c.close()


@pytest.fixture(scope="module", params=[(0, 0), (3, 0), (0, 1)], ids=["k_match", "k_win_mma", "k_describe_tiled"])
def wctx(request, brief_pattern):
    """The windowed matcher with its distances from k_match (matcher 0) and
    from the tensor cores (matcher 3), and the describe stage reading its
    tests from TMA-staged shared-memory boxes (describe_form 1): the same
    features and lists."""
    matcher, form = request.param
    c = Context(brief_pattern, levels=6, max_width=1280, max_height=720, matcher=matcher, describe_form=form)
    yield c
    c.close()


def _run(ctx, frames, pairs=()):
    b = Batch(ctx, [(f.shape[1], f.shape[0]) for f in frames], list(pairs))
    b.process(frames)
    return b


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def _assert_features_equal(got, exp):
    gf, gk, gr = got
    ef, ek, er = exp
    assert np.array_equal(gr, er), (gr, er)
    assert np.array_equal(gk, ek), (gk, ek)
    assert gf.shape == ef.shape
    if gf.tobytes() != ef.tobytes():
        gb = gf.view(np.uint8).reshape(len(gf), 48)
        eb = ef.view(np.uint8).reshape(len(ef), 48)
        bad = np.nonzero((gb != eb).any(1))[0]
        i = int(bad[0])
        raise AssertionError(f"{len(bad)} feature records differ; first #{i}: gpu={gf[i]} oracle={ef[i]}")


def test_pyramid_levels_bit_exact(ctx):
    f1, _ = synth.warped_pair(0)
    b = _run(ctx, [f1])
    try:
        for l in range(1, 6):
            assert np.array_equal(b.pyramid_level(0, l).view(np.uint32),
                                  oracle.pyramid_level(f1, l).view(np.uint32)), f"level {l}"
    finally:
        b.close()


def test_blur_cache_bit_exact(ctx):
    f1, _ = synth.warped_pair(1)
    b = _run(ctx, [f1])
    try:
        for l in range(6):
            exp = oracle.blur_level(oracle.pyramid_level(f1, l))
            assert np.array_equal(b.blur_level(0, l).view(np.uint32), exp.view(np.uint32)), f"level {l}"
    finally:
        b.close()


def test_blur_cache_border_bit_exact(ctx):
    """Cells beyond the level edge and the negative-coordinate sentinels hold
    G(P) of generate_features.wgsl:149-172 at those points (u32-wrapped)."""
    f1, _ = synth.warped_pair(2)
    m = ctx.blur_margin()
    b = _run(ctx, [f1])
    try:
        for l in (2, 5):
            lvl = oracle.pyramid_level(f1, l)
            h, w = lvl.shape
            ext = b.blur_level(0, l, extended=True)
            assert ext.shape == (h + m + 1, w + m + 1)
            for ey in range(h + m + 1):
                py = ey if ey < h + m else 0xFFFFFFFF
                xs = range(w + m + 1) if ey >= h else range(w, w + m + 1)
                for ex in xs:
                    px = ex if ex < w + m else 0xFFFFFFFF
                    exp = np.float32(oracle.gauss_tap9(lvl, px, py))
                    assert ext[ey, ex].view(np.uint32) == exp.view(np.uint32), (l, ex, ey)
            # every negative coordinate the pattern can reach maps to the sentinel
            for k in (1, 7, m - 1):
                assert np.float32(oracle.gauss_tap9(lvl, (-k) & 0xFFFFFFFF, 5)).view(np.uint32) == \
                    ext[5, w + m].view(np.uint32)
    finally:
        b.close()


def test_keypoint_maps_bit_exact(ctx):
    for seed in (0, 3):
        f1, _ = synth.warped_pair(seed)
        b = _run(ctx, [f1])
        try:
            for l in range(6):
                lvl = oracle.pyramid_level(f1, l)
                exp = oracle.cull(oracle.detect(lvl), 752, 480)
                assert np.array_equal(b.keypoint_map(0, l).astype(np.uint32), exp), f"seed {seed} level {l}"
        finally:
            b.close()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_features_and_matches_bit_exact(ctx, brief_pattern, seed):
    f1, f2 = synth.warped_pair(seed)
    b = _run(ctx, [f1, f2], [(0, 1)])
    try:
        got = [b.features(i) for i in range(2)]
        exp = [oracle.frame(f, brief_pattern) for f in (f1, f2)]
        for g, e in zip(got, exp):
            _assert_features_equal(g, e)
        em = oracle.match(exp[0][0], exp[0][1], exp[1][0], exp[1][1], 752, 480)
        gm = _mm(b.matches(0))
        assert len(em) > 100
        assert np.array_equal(gm, em)
        ref = oracle.ref_matcher(752, 480)
        # the reference's own compiled matcher: built wherever its source (or the
        # copy staged beside the repository) is at hand
        assert ref is not None or not oracle.ref_matcher_expected()
        if ref is not None:
            assert np.array_equal(gm, ref(exp[0][0], exp[0][1], exp[1][0], exp[1][1]))
    finally:
        b.close()


def test_uneven_batch_equals_oracle_and_alone(wctx, brief_pattern):
    sizes = [(640, 480), (752, 480), (1280, 720), (97, 61), (333, 211)]
    frames, pairs = [], []
    for k, (w, h) in enumerate(sizes):
        a, c = synth.warped_pair(100 + k, w, h)
        frames += [a, c]
        pairs.append((2 * k, 2 * k + 1))
    ctx = wctx
    b = _run(ctx, frames, pairs)
    try:
        for k, (w, h) in enumerate(sizes):
            exp = [oracle.frame(frames[2 * k + j], brief_pattern) for j in range(2)]
            for j in range(2):
                _assert_features_equal(b.features(2 * k + j), exp[j])
            em = oracle.match(exp[0][0], exp[0][1], exp[1][0], exp[1][1], w, h)
            assert np.array_equal(_mm(b.matches(k)), em), f"pair {k} {w}x{h}"
        # the same pair alone in its own batch gives the same bytes
        alone = _run(ctx, frames[4:6], [(0, 1)])
        try:
            assert alone.features(1)[0].tobytes() == b.features(5)[0].tobytes()
            assert np.array_equal(_mm(alone.matches(0)), _mm(b.matches(2)))
        finally:
            alone.close()
    finally:
        b.close()


def test_repeat_runs_are_identical(ctx):
    frames = synth.plane_sequence(5, n=4)
    b = Batch(ctx, [(752, 480)] * 4, [(0, 1), (1, 2), (2, 3)])
    try:
        b.process(frames)
        first = [b.features(i)[0].tobytes() for i in range(4)] + [_mm(b.matches(p)).tobytes() for p in range(3)]
        b.run()
        b.download()
        b.sync()
        again = [b.features(i)[0].tobytes() for i in range(4)] + [_mm(b.matches(p)).tobytes() for p in range(3)]
        assert first == again
    finally:
        b.close()


def test_constant_and_tiny_frames(brief_pattern):
    with Context(brief_pattern, levels=6, max_width=64, max_height=64, cap_per_level=50) as c:
        flat = np.full((48, 64), 77, np.uint8)
        tiny = synth.scene_frame(9, 10, 10)
        odd = synth.scene_frame(11, 37, 23)
        frames = [flat, flat, tiny, tiny, odd]
        b = _run(c, frames, [(0, 1), (2, 3)])
        try:
            f, kept, raw = b.features(0)
            assert len(f) == 0 and not raw.any()
            assert len(b.matches(0)) == 0
            for i in (2, 4):
                _assert_features_equal(b.features(i), oracle.frame(frames[i], brief_pattern, cap=50))
        finally:
            b.close()


def test_widest_tallest_frames_and_most_levels(brief_pattern):
    """The largest frame width the context accepts (8192) and a frame of that
    height, each as a warped pair, with the most pyramid levels (12; level 11
    is 1102 x 12 or 12 x 1102): bit-exact against the oracle."""
    with Context(brief_pattern, levels=12, max_width=8192, max_height=8192) as c:
        frames = list(synth.warped_pair(21, 8192, 96)) + list(synth.warped_pair(22, 96, 8192))
        b = _run(c, frames, [(0, 1), (2, 3)])
        try:
            for k, (w, h) in enumerate([(8192, 96), (96, 8192)]):
                exp = [oracle.frame(frames[2 * k + j], brief_pattern, levels=12) for j in range(2)]
                for j in range(2):
                    _assert_features_equal(b.features(2 * k + j), exp[j])
                    assert exp[j][1][11] > 0, "no feature on the smallest level"
                em = oracle.match(exp[0][0], exp[0][1], exp[1][0], exp[1][1], w, h)
                assert len(em) > 0
                assert np.array_equal(_mm(b.matches(k)), em), f"pair {k} {w}x{h}"
        finally:
            b.close()


def test_tiled_describe_edge_frames(brief_pattern):
    """With describe_form 1, batches of 8 frames or more describe over
    blur-cache boxes staged in shared memory (k_describe_tiled).  The edge cases in one such batch: the
    widest and tallest frames (8192 x 96, 96 x 8192, 12 levels: 64 column
    chunks, 256 bands), tiny and odd frames whose boxes reach past every
    edge (tests at negative coordinates read the sentinels), and a constant
    frame; all bit-exact against the oracle."""
    with Context(brief_pattern, levels=12, max_width=8192, max_height=8192, describe_form=1) as c:
        frames = list(synth.warped_pair(21, 8192, 96)) + list(synth.warped_pair(22, 96, 8192))
        frames += [synth.scene_frame(9, 10, 10), synth.scene_frame(11, 37, 23), synth.scene_frame(12, 61, 45),
                   np.full((48, 64), 77, np.uint8)]
        assert len(frames) >= 8
        b = _run(c, frames, [(0, 1), (2, 3)])
        try:
            exp = [oracle.frame(f, brief_pattern, levels=12) for f in frames]
            for i in range(len(frames)):
                _assert_features_equal(b.features(i), exp[i])
            for k, (w, h) in enumerate([(8192, 96), (96, 8192)]):
                em = oracle.match(exp[2 * k][0], exp[2 * k][1], exp[2 * k + 1][0], exp[2 * k + 1][1], w, h)
                assert len(em) > 0
                assert np.array_equal(_mm(b.matches(k)), em), f"pair {k} {w}x{h}"
            assert sum(int(e[1].sum()) for e in exp[4:7]) > 0
        finally:
            b.close()


def test_cap_keeps_first_in_yx_order(brief_pattern):
    f1, _ = synth.warped_pair(4)
    with Context(brief_pattern, levels=6, max_width=752, max_height=480, cap_per_level=100) as c:
        b = _run(c, [f1])
        try:
            got = b.features(0)
            exp = oracle.frame(f1, brief_pattern, cap=100)
            _assert_features_equal(got, exp)
            assert (got[1] == 100).all() and (got[2] > 100).all()
        finally:
            b.close()


def test_frontend_rotation_matches_reference_rule(ctx, brief_pattern):
    """FeatureSet(1) advances on the marker or when absent
    (load_features_cpu.cpp:111-142); matching is FeatureSet(1) -> FeatureSet(0)."""
    frames = synth.plane_sequence(7, n=6)
    advance = [False, False, False, True, False, True]
    fe = Frontend(ctx, 752, 480)
    try:
        ref_set = None
        cur_set = None
        for i, (img, adv) in enumerate(zip(frames, advance)):
            matched = fe.process(img, advance_reference=adv)
            exp = oracle.frame(img, brief_pattern)
            if cur_set is not None and (ref_set is None or adv):
                ref_set = cur_set
            cur_set = exp
            assert matched == (ref_set is not None)
            _assert_features_equal(fe.features(0), exp)
            if ref_set is not None:
                _assert_features_equal(fe.features(1), ref_set)
                em = oracle.match(ref_set[0], ref_set[1], exp[0], exp[1], 752, 480)
                assert np.array_equal(_mm(fe.matches()), em), f"frame {i}"
    finally:
        fe.close()


def test_large_batch_bit_exact(wctx, brief_pattern):
    """22 frames (~170k keypoints, larger describe groups than the small
    tests), captured as two halves on two streams: every frame's features and
    a pair within the second half equal the oracle."""
    frames = synth.plane_sequence(77, n=22)
    b = _run(wctx, frames, [(i, i + 1) for i in range(len(frames) - 1)])
    try:
        total = 0
        for i, f in enumerate(frames):
            exp = oracle.frame(f, brief_pattern)
            _assert_features_equal(b.features(i), exp)
            total += int(exp[1].sum())
        assert total > 160_000
        a, c = oracle.frame(frames[20], brief_pattern), oracle.frame(frames[21], brief_pattern)
        em = oracle.match(a[0], a[1], c[0], c[1], 752, 480)
        assert np.array_equal(_mm(b.matches(20)), em)
    finally:
        b.close()


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("matcher", [0, 2, 3])
def test_split_batch_pairs_across_halves(brief_pattern, matcher, form):
    """A batch of 20 frames is captured as two halves (frames 0-9 and 10-19)
    on two streams.  Pairs within either half, from the first half into the
    second and from the second back into the first all equal the oracle, with
    the windowed matcher (distances from k_match or from the tensor cores) and
    with the tensor-core brute-force matcher, each with either describe form
    (the tiled form also writing the matchers' operand rows)."""
    W, H = 320, 240
    frames = [synth.scene_frame(300 + k, W, H) for k in range(20)]
    pairs = [(0, 1), (3, 12), (15, 2), (10, 11), (19, 0), (9, 10), (8, 9), (12, 19)]
    with Context(brief_pattern, levels=6, max_width=W, max_height=H, matcher=matcher, ratio=0.8,
                 describe_form=form) as c:
        b = Batch(c, [(W, H)] * len(frames), pairs)
        try:
            b.process(frames)
            exp = [oracle.frame(f, brief_pattern) for f in frames]
            for i in range(len(frames)):
                _assert_features_equal(b.features(i), exp[i])
            for k, (p, q) in enumerate(pairs):
                if matcher in (0, 3):
                    em = oracle.match(exp[p][0], exp[p][1], exp[q][0], exp[q][1], W, H)
                else:
                    em = oracle.match_bruteforce(exp[p][0], exp[p][1], exp[q][0], exp[q][1], 0.8)
                assert np.array_equal(_mm(b.matches(k)), em), (matcher, k, p, q)
            assert sum(len(b.matches(k)) for k in range(len(pairs))) > 50
        finally:
            b.close()
