"""Brute-force top-2 matchers against the oracle: matcher 1 (XOR + popcount
on the integer pipes) and matcher 2 (distances from FP8 dot products on the
tensor cores, tcgen05), which must give identical match lists.  The full
match list at 752x480 and on an uneven batch, and at the 3840x2160, 8-level,
2500-per-level stress size (20000 x 20000 descriptors) as well."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import Batch, Context, synth

pytestmark = pytest.mark.gpu


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


@pytest.mark.parametrize("matcher", [1, 2])
def test_bruteforce_equals_oracle_uneven(brief_pattern, matcher):
    frames = list(synth.warped_pair(5)) + list(synth.warped_pair(6, 1280, 720)) + [
        np.full((480, 640), 77, np.uint8), synth.scene_frame(9, 640, 480)]
    pairs = [(0, 1), (2, 3), (4, 5), (5, 4), (1, 0)]
    with Context(brief_pattern, levels=6, max_width=1280, max_height=720, matcher=matcher, ratio=0.8) as c:
        b = Batch(c, [(f.shape[1], f.shape[0]) for f in frames], pairs)
        try:
            b.process(frames)
            exp = [oracle.frame(f, brief_pattern) for f in frames]
            for i in range(len(frames)):
                gf, gk, _ = b.features(i)
                assert gf.tobytes() == exp[i][0].tobytes() and np.array_equal(gk, exp[i][1])
            for k, (p, q) in enumerate(pairs):
                em = oracle.match_bruteforce(exp[p][0], exp[p][1], exp[q][0], exp[q][1], 0.8)
                assert np.array_equal(_mm(b.matches(k)), em), f"pair {k}"
            assert len(_mm(b.matches(0))) > 200
            assert len(_mm(b.matches(2))) == 0  # constant frame: no features
        finally:
            b.close()


@pytest.mark.parametrize("matcher", [1, 2])
def test_bruteforce_stress_size(brief_pattern, matcher):
    W, H, L, CAP = 3840, 2160, 8, 2500
    f0, f1 = synth.warped_pair(2024, W, H, n_rect=5000, n_check=500, scale_by_area=False)
    with Context(brief_pattern, levels=L, max_width=W, max_height=H, cap_per_level=CAP, matcher=matcher,
                 ratio=0.8) as c:
        b = Batch(c, [(W, H), (W, H)], [(0, 1)])
        try:
            b.process([f0, f1])
            ea = oracle.frame(f0, brief_pattern, levels=L, cap=CAP)
            eb = oracle.frame(f1, brief_pattern, levels=L, cap=CAP)
            for i, e in enumerate((ea, eb)):
                gf, gk, gr = b.features(i)
                assert np.array_equal(gk, e[1]) and np.array_equal(gr, e[2])
                assert gf.tobytes() == e[0].tobytes()
            assert ea[1].sum() > 15000 and eb[1].sum() > 15000
            em = oracle.match_bruteforce(ea[0], ea[1], eb[0], eb[1], 0.8)
            assert np.array_equal(_mm(b.matches(0)), em)
            assert len(em) > 1000
        finally:
            b.close()


@pytest.mark.parametrize("matcher", [1, 2])
def test_bruteforce_split_and_unsplit_agree(brief_pattern, matcher):
    """A launch with few pairs splits each train set over several CTAs and
    merges the partial top-2 records; a launch with many query blocks (large
    per-level caps) does not split.  Both equal the oracle."""
    pairs_frames = [synth.warped_pair(130 + k, 640, 480) for k in range(3)]
    frames = [f for pr in pairs_frames for f in pr]
    pairs = [(2 * k, 2 * k + 1) for k in range(3)]
    exp = [oracle.frame(f, brief_pattern, cap=20000) for f in frames]
    for cap in (20000, 1000):  # 3 x 469 query blocks: no split; 3 x 24: split
        with Context(brief_pattern, levels=6, max_width=640, max_height=480, cap_per_level=cap, matcher=matcher,
                     ratio=0.8) as c:
            b = Batch(c, [(640, 480)] * len(frames), pairs)
            try:
                b.process(frames)
                for k, (p, q) in enumerate(pairs):
                    ep = exp[p] if cap == 20000 else oracle.frame(frames[p], brief_pattern, cap=cap)
                    eq = exp[q] if cap == 20000 else oracle.frame(frames[q], brief_pattern, cap=cap)
                    em = oracle.match_bruteforce(ep[0], ep[1], eq[0], eq[1], 0.8)
                    assert np.array_equal(_mm(b.matches(k)), em), (cap, k)
                    assert len(em) > 50
            finally:
                b.close()


@pytest.mark.parametrize("matcher", [0, 1, 2, 3])
def test_single_feature_sets(brief_pattern, matcher):
    """Frames with exactly one feature (one bright pixel on a flat frame: at
    (297, 262) it survives on level 0 only, at (579, 137) on level 1 only):
    a train set or pool of one feature gives no match (fewer than two,
    match_features_cpu.cpp:80-82), and a single query finds its own feature
    in a train set of two.  For matcher 2 the train rows sit in a 128-row tile
    whose other rows are not features."""
    W, H = 640, 480
    one_a = np.full((H, W), 128, np.uint8)
    one_a[262, 297] = 255
    one_b = np.full((H, W), 128, np.uint8)
    one_b[137, 579] = 255
    full = synth.scene_frame(9, W, H)
    two = one_a.copy()  # both pixels: both features
    two[137, 579] = 255
    frames = [one_a, one_b, full, two]
    pairs = [(0, 2), (2, 0), (0, 1), (1, 0), (2, 1), (0, 3), (3, 0)]
    with Context(brief_pattern, levels=6, max_width=W, max_height=H, matcher=matcher, ratio=0.8) as c:
        b = Batch(c, [(W, H)] * len(frames), pairs)
        try:
            b.process(frames)
            exp = [oracle.frame(f, brief_pattern) for f in frames]
            assert exp[0][1].tolist() == [1, 0, 0, 0, 0, 0] and exp[1][1].tolist() == [0, 1, 0, 0, 0, 0]
            assert exp[3][1].tolist() == [1, 1, 0, 0, 0, 0]
            for i in range(len(frames)):
                gf, gk, _ = b.features(i)
                assert gf.tobytes() == exp[i][0].tobytes() and np.array_equal(gk, exp[i][1])
            for k, (p, q) in enumerate(pairs):
                if matcher in (0, 3):
                    em = oracle.match(exp[p][0], exp[p][1], exp[q][0], exp[q][1], W, H)
                else:
                    em = oracle.match_bruteforce(exp[p][0], exp[p][1], exp[q][0], exp[q][1], 0.8)
                    if len(exp[q][0]) < 2:
                        assert len(em) == 0
                assert np.array_equal(_mm(b.matches(k)), em), f"pair {k}"
            if matcher in (1, 2):  # the single query finds itself among two train features
                assert len(_mm(b.matches(5))) == 1
        finally:
            b.close()


@pytest.mark.parametrize("matcher", [0, 1, 2, 3])
def test_tied_best_is_rejected(brief_pattern, matcher):
    """Exact ties: frame B1 holds two features whose descriptors both equal
    the single feature of frame A (bright pixels at (297, 262) and (315, 262)
    on a flat frame), so a query for that descriptor meets two candidates at
    distance 0 and the ratio test rejects it (best == second;
    match_features_cpu.cpp:133-146).  B2 (second pixel at (324, 262)) has a
    different second descriptor and matches.  All 12 ordered pairs of
    A, B1, B2 and C (A plus a far feature) equal the oracle."""
    W, H = 640, 480
    base = np.full((H, W), 128, np.uint8)
    base[262, 297] = 255
    b1, b2, cc = base.copy(), base.copy(), base.copy()
    b1[262, 315] = 255
    b2[262, 324] = 255
    cc[137, 579] = 255
    frames = [base, b1, b2, cc]
    pairs = [(p, q) for p in range(4) for q in range(4) if p != q]
    with Context(brief_pattern, levels=6, max_width=W, max_height=H, matcher=matcher, ratio=0.8) as c:
        b = Batch(c, [(W, H)] * len(frames), pairs)
        try:
            b.process(frames)
            exp = [oracle.frame(f, brief_pattern) for f in frames]
            d = exp[1][0]["descriptor"]
            assert exp[1][1].tolist() == [2, 0, 0, 0, 0, 0] and (d == exp[0][0]["descriptor"][0]).all()
            got = {}
            for k, (p, q) in enumerate(pairs):
                if matcher in (0, 3):
                    em = oracle.match(exp[p][0], exp[p][1], exp[q][0], exp[q][1], W, H)
                else:
                    em = oracle.match_bruteforce(exp[p][0], exp[p][1], exp[q][0], exp[q][1], 0.8)
                g = _mm(b.matches(k))
                assert np.array_equal(g, em), f"pair {p}->{q}"
                got[(p, q)] = len(g)
            if matcher in (0, 3):  # C -> B1 tied (no mutual pair), C -> B2 not
                assert got[(3, 1)] == 0 and got[(3, 2)] == 1
            else:  # A -> B1 tied, A -> B2 not
                assert got[(0, 1)] == 0 and got[(0, 2)] == 1
        finally:
            b.close()


def test_tensor_core_matcher_pair_limit(brief_pattern):
    """Matcher 2 keeps its per-launch unit table in shared memory: a batch
    with more than 1024 pairs is refused with CAPACITY at creation, and 1024
    pairs are accepted."""
    from uni_slam_gb300 import USlamError, capi

    with Context(brief_pattern, levels=2, max_width=64, max_height=64, matcher=2, ratio=0.8) as c:
        for n, ok in ((1024, True), (1025, False)):
            sizes = [(64, 64)] * (n + 1)
            pairs = [(i, i + 1) for i in range(n)]
            if ok:
                Batch(c, sizes, pairs).close()
            else:
                with pytest.raises(USlamError) as ei:
                    Batch(c, sizes, pairs)
                assert ei.value.status == capi.CAPACITY
