"""The library's closed-form culling (coverage bitmap + row-0 arg-max) equals
the oracle's literal simulation of both cull dispatches, with the index bugs
of resources/cull_corners.wgsl, for every level of every configured size."""
import numpy as np
import pytest

import oracle
from uni_slam_gb300 import capi


def _coverage(W0, H0, w, h):
    lib = capi.load()
    bits = np.zeros((w * h + 31) // 32, np.uint32)
    assert lib.uslam_cull_coverage(W0, H0, w, h, capi.ptr(bits)) == capi.OK
    m = np.unpackbits(bits.view(np.uint8), bitorder="little")[: w * h]
    return m.reshape(h, w).astype(bool)


def _apply(resp, cov):
    h, w = resp.shape
    out = np.where(cov & (resp > 0), resp, 0).astype(np.uint32)
    row = resp[0]
    for x in range(w):
        if out[0, x] == 0:
            continue
        start = x - x % 9
        end = min(start + 3, w)
        for q in range(start, end):
            if (q < x and row[q] >= row[x]) or (q > x and row[q] > row[x]):
                out[0, x] = 0
    return out


@pytest.mark.parametrize("size", [(752, 480), (640, 480), (1280, 720), (64, 48), (10, 10), (97, 61)])
def test_coverage_equals_literal_cull(size):
    W0, H0 = size
    rs = np.random.RandomState(W0 * 7 + H0)
    for l, (w, h) in enumerate(oracle.level_dims(W0, H0, 6)):
        cov = _coverage(W0, H0, w, h)
        for density in (0.05, 0.5, 1.0):
            resp = np.where(rs.uniform(size=(h, w)) < density, rs.randint(10, 18, size=(h, w)), 0).astype(np.uint32)
            assert np.array_equal(_apply(resp, cov), oracle.cull(resp, W0, H0)), (size, l, density)


def test_row0_keypoints_only_at_multiples_of_9():
    cov = _coverage(752, 480, 752, 480)
    xs = np.nonzero(cov[0])[0]
    assert (xs % 9 == 0).all() and len(xs) == len(range(0, 752, 9))
