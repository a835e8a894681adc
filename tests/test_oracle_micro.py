"""Hand-computed micro-cases for the CPU restatement of the WGSL passes
(resources/*.wgsl).  The reference ships no golden vectors for these passes
and cannot run them (no Dawn, no graphics stack), so these known answers
are the pins the oracle's detect / cull / describe logic rests on."""
import numpy as np

import oracle


def test_level_dims_table():
    # wslam/src/common.cpp:41-45 — the per-configuration table
    assert oracle.level_dims(752, 480) == [(752, 480), (626, 400), (522, 333), (435, 277), (362, 231), (302, 192)]
    assert oracle.level_dims(640, 480) == [(640, 480), (533, 400), (444, 333), (370, 277), (308, 231), (257, 192)]
    assert oracle.level_dims(1280, 720) == [(1280, 720), (1066, 600), (888, 500), (740, 416), (617, 347), (514, 289)]
    assert oracle.level_dims(1920, 1080) == [(1920, 1080), (1600, 900), (1333, 750), (1111, 625), (925, 520),
                                             (771, 434)]
    d8 = oracle.level_dims(3840, 2160, 8)
    assert d8[5] == (1543, 868) and d8[6] == (1286, 723) and d8[7] == (1071, 602)
    assert sum(w * h for w, h in oracle.level_dims(752, 480)) == 1047287


def test_lod0_threshold_is_integer_rule():
    # |a/255 - b/255| > 0.15f  <=>  |a - b| >= 39, for all 256^2 pairs
    a = np.arange(256, dtype=np.float32) / np.float32(255.0)
    d = np.abs(a[:, None] - a[None, :]) > np.float32(0.15)
    ia = np.arange(256)
    assert np.array_equal(d, np.abs(ia[:, None] - ia[None, :]) >= 39)


def test_constant_image_has_no_response():
    lvl = np.full((40, 50), 0.5, np.float32)
    assert not oracle.detect(lvl).any()


def test_isolated_bright_pixel_response_is_17():
    # every circle pixel differs: run of 16 -> response 1 + 16 = 17
    lvl = np.zeros((20, 20), np.float32)
    lvl[10, 10] = 1.0
    r = oracle.detect(lvl)
    assert r[10, 10] == 17
    # pixels at distance 3 see the bright pixel once on their circle: run 1
    assert r[10, 13] == 0


def test_bright_square_corner_response():
    # a bright square occupying x, y >= 10: the outer corner pixel (10, 10)
    # sees circle points i = 3..7 (x >= 10 and y >= 10 fail for the others).
    lvl = np.zeros((30, 30), np.float32)
    lvl[10:, 10:] = 1.0
    r = oracle.detect(lvl)
    # corner pixel is bright; circle points with dx<0 or dy<0 are dark -> differ.
    cx = [0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3, -3, -3, -2, -1]
    cy = [-3, -3, -2, -1, 0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3]
    diff = [(dx < 0 or dy < 0) for dx, dy in zip(cx, cy)]
    run = best = 0
    for d in diff:
        run = run + 1 if d else 0
        best = max(best, run)
    expect = best + 1 if best + 1 > 9 else 0
    assert r[10, 10] == expect


def test_negative_coordinates_read_far_edge():
    # Tint clamp: a negative coordinate reads row/column n-1.  At pixel (0, 0)
    # every circle point with dx < 0 or dy < 0 lands on the last column/row,
    # which are bright; the in-range circle points are set bright too, so all
    # 16 differ from the dark centre -> response 17.  A clamp to 0 would read
    # the dark centre for those points instead.
    lvl = np.zeros((16, 16), np.float32)
    lvl[15, :] = 1.0
    lvl[:, 15] = 1.0
    for x, y in [(3, 0), (3, 1), (2, 2), (1, 3), (0, 3)]:
        lvl[y, x] = 1.0
    assert oracle.detect(lvl)[0, 0] == 17


def test_cull_row0_first_argmax_and_stride():
    W0, H0 = 64, 48
    resp = np.zeros((H0, W0), np.uint32)
    resp[0, 9:12] = [12, 15, 15]     # region [9, 12): first arg-max at 10
    resp[0, 18:21] = [0, 0, 11]      # region [18, 21): max at 20
    resp[0, 3] = 17                  # outside any region start set -> dropped
    out = oracle.cull(resp, W0, H0)
    # row 0 also needs the vertical pass, which only covers multiples of 3
    assert out[0, 10] == 0 and out[0, 9] == 0  # 10 % 3 != 0: dropped by V
    assert out[0, 3] == 0
    assert out[0, 18] == 0 and out[0, 20] == 0
    resp2 = np.zeros((H0, W0), np.uint32)
    resp2[0, 27:30] = [16, 12, 10]   # first arg-max at 27 (multiple of 9 and 3)
    out2 = oracle.cull(resp2, W0, H0)
    assert out2[0, 27] == 16 and out2[0, 28] == 0


def test_cull_is_a_mask_for_rows_after_zero():
    rs = np.random.RandomState(3)
    W0, H0 = 752, 480
    resp = np.where(rs.uniform(size=(H0, W0)) < 0.5, rs.randint(10, 18, size=(H0, W0)), 0).astype(np.uint32)
    out = oracle.cull(resp, W0, H0)
    sub = out[1:] > 0
    # every surviving pixel keeps its response value unchanged
    assert np.array_equal(out[1:][sub], resp[1:][sub])
    # doubling the density cannot add survivors at pixels without response
    assert not (out[1:][resp[1:] == 0]).any()


def test_describe_constant_patch_all_zero_bits():
    lvl = np.full((64, 64), 0.25, np.float32)
    pat = np.random.RandomState(0).randint(-13, 13, size=(256, 4)).astype(np.int32)
    th, d = oracle.describe(lvl, 32, 32, pat)
    assert th == 0.0           # atan2(0, 0) = +0
    assert not d.any()         # G(A) > G(B) never holds on a flat level


def test_gauss_tap9_flat_interior():
    lvl = np.full((32, 32), 0.5, np.float32)
    # weights sum to 1 in f32 arithmetic up to rounding
    assert abs(oracle.gauss_tap9(lvl, 16, 16) - 0.5) < 1e-6
